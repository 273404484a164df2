// Host side of libmorgana_gpu.so: error state, quadrature and reference-element
// tables, mesh ingest, edge and dof numbering.
//
// Reference behaviour restated here (paths relative to the morganaPublic checkout):
//   quadrature points/weights  src/morganaIntegrator/intStaticCards.cpp:707-991
//   P1/P2 basis                src/morganaPolynomial/polyCards.cpp:232-285
//   Gmsh 2 ingest              src/morganaFile/loadMesh.hpp:2065-2330
//   Jacobian check             src/morganaGeometry/meshDoctor3d.hpp:195-227
//   edges                      src/morganaGeometry/connect3d.hpp:417-491,
//                              src/morganaGeometry/geoShapes.cpp:670-677
//   edge numbering             src/morganaContainer/pVectGlobalManip.hpp:414-578
//   dof numbering              src/morganaFields/dofMapStatic3d.hpp:420-662
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "mg_internal.h"

namespace mg {

// ------------------------------------------------------------------ errors --
static thread_local std::string g_last_error;

mg_status set_error(mg_status s, const std::string& msg)
{
  g_last_error = msg;
  return s;
}

mg_status cuda_error(cudaError_t e, const char* what)
{
  return set_error(e == cudaErrorMemoryAllocation ? MG_ERR_ALLOC : MG_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

// -------------------------------------------------------------- quadrature --
// The four linearTetra STANDARD cards of the reference (same decimal constants,
// which matter for the 64-point card: they are rounded to 10 digits) and the
// 11-point degree-4 rule of Keast (1986), built from its closed forms.
int quad_rule(int quad, std::vector<double>* Y, std::vector<double>* W)
{
  Y->clear();
  W->clear();
  auto add = [&](double x, double y, double z, double w) {
    Y->push_back(x); Y->push_back(y); Y->push_back(z); W->push_back(w);
  };
  switch (quad) {
    case 1:
      add(0.25, 0.25, 0.25, 1.0 / 6.0);
      break;
    case 4: {
      const double a = (5.0 - std::sqrt(5.0)) / 20.0, b = (5.0 + 3 * std::sqrt(5.0)) / 20.0;
      add(a, a, a, 1.0 / 24.0);
      add(a, a, b, 1.0 / 24.0);
      add(a, b, a, 1.0 / 24.0);
      add(b, a, a, 1.0 / 24.0);
      break;
    }
    case 11: {
      // barycentric orbits: centroid; (1/14,1/14,1/14,11/14); (a,a,b,b)
      const double c = 0.25, p = 1.0 / 14.0, q = 11.0 / 14.0;
      const double a = (1.0 + std::sqrt(5.0 / 14.0)) / 4.0, b = (1.0 - std::sqrt(5.0 / 14.0)) / 4.0;
      const double w0 = -74.0 / 5625.0, w1 = 343.0 / 45000.0, w2 = 56.0 / 2250.0;
      add(c, c, c, w0);
      add(p, p, p, w1); add(q, p, p, w1); add(p, q, p, w1); add(p, p, q, w1);
      add(a, a, b, w2); add(a, b, a, w2); add(b, a, a, w2);
      add(b, b, a, w2); add(b, a, b, w2); add(a, b, b, w2);
      break;
    }
    case 15: {
      const double r5 = 0.25;
      const double s5[2] = {0.09197107805272303, 0.3197936278296299};
      const double t5[2] = {0.7240867658418310, 0.04061911651111023};
      const double u5 = 0.05635083268962915, v5 = 0.4436491673103708;
      const double A5 = 0.01975308641975309, C5 = 0.008818342151675485;
      const double B5[2] = {0.01198951396316977, 0.01151136787104540};
      add(r5, r5, r5, A5);
      for (int k = 0; k < 2; ++k) {
        add(s5[k], s5[k], s5[k], B5[k]);
        add(t5[k], s5[k], s5[k], B5[k]);
        add(s5[k], t5[k], s5[k], B5[k]);
        add(s5[k], s5[k], t5[k], B5[k]);
      }
      add(u5, u5, v5, C5); add(u5, v5, u5, C5); add(v5, u5, u5, C5);
      add(v5, v5, u5, C5); add(v5, u5, v5, C5); add(u5, v5, v5, C5);
      break;
    }
    case 64: {
      const double t[4] = {0.0485005494, 0.2386007376, 0.5170472951, 0.7958514179};
      const double s[4] = {0.0571041961, 0.2768430136, 0.5835904324, 0.8602401357};
      const double r[4] = {0.0694318422, 0.3300094782, 0.6699905218, 0.9305681558};
      const double A[4] = {0.1739274226, 0.3260725774, 0.3260725774, 0.1739274226};
      const double B[4] = {0.1355069134, 0.2034645680, 0.1298475476, 0.0311809709};
      const double C[4] = {0.1108884156, 0.1434587898, 0.0686338872, 0.0103522407};
      // conical product: r (Gauss-Legendre, weights A), s (weights B), t (weights C)
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          for (int k = 0; k < 4; ++k)
            add(t[k], s[j] * (1 - t[k]), r[i] * (1 - s[j]) * (1 - t[k]), A[i] * B[j] * C[k]);
      break;
    }
    default:
      return 0;
  }
  return (int)W->size();
}

// ------------------------------------------------------------------- basis --
// Barycentric form: l0 = 1-x-y-z, l1 = x, l2 = y, l3 = z.  P2 vertex functions
// l_i(2 l_i - 1), edge functions 4 l_a l_b over the reference's local edge order
// (1,2),(2,3),(3,1),(1,4),(2,4),(3,4).
static const int kEdgePts[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
static const double kGradL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

void basis_values(int order, const double* Y, double* v)
{
  const double l[4] = {1.0 - Y[0] - Y[1] - Y[2], Y[0], Y[1], Y[2]};
  if (order == 1) {
    for (int i = 0; i < 4; ++i) v[i] = l[i];
    return;
  }
  for (int i = 0; i < 4; ++i) v[i] = l[i] * (2.0 * l[i] - 1.0);
  for (int j = 0; j < 6; ++j) v[4 + j] = 4.0 * l[kEdgePts[j][0]] * l[kEdgePts[j][1]];
}

void basis_grads(int order, const double* Y, double* gx, double* gy, double* gz)
{
  double* g[3] = {gx, gy, gz};
  const double l[4] = {1.0 - Y[0] - Y[1] - Y[2], Y[0], Y[1], Y[2]};
  if (order == 1) {
    for (int i = 0; i < 4; ++i)
      for (int c = 0; c < 3; ++c) g[c][i] = kGradL[i][c];
    return;
  }
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 3; ++c) g[c][i] = (4.0 * l[i] - 1.0) * kGradL[i][c];
  for (int j = 0; j < 6; ++j) {
    const int a = kEdgePts[j][0], b = kEdgePts[j][1];
    for (int c = 0; c < 3; ++c) g[c][4 + j] = 4.0 * (l[a] * kGradL[b][c] + l[b] * kGradL[a][c]);
  }
}

mg_status build_ref_tables(int order, int quad, RefTables* t)
{
  std::vector<double> Y, W;
  const int nq = quad_rule(quad, &Y, &W);
  if (nq == 0) return set_error(MG_ERR_INVALID_ARG, "unknown quadrature rule " + std::to_string(quad));
  const int nb = nbasis(order);
  t->order = order;
  t->quad = quad;
  t->nb = nb;
  t->nq = nq;
  t->stiff.assign(6 * nb * nb, 0.0);
  t->mass.assign(nb * nb, 0.0);
  t->wsum = 0.0;
  static const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
  for (int q = 0; q < nq; ++q) {
    double v[10], gx[10], gy[10], gz[10];
    basis_values(order, &Y[3 * q], v);
    basis_grads(order, &Y[3 * q], gx, gy, gz);
    const double* g[3] = {gx, gy, gz};
    const double w = W[q];
    t->wsum += w;
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        t->mass[i * nb + j] += w * v[i] * v[j];
        for (int p = 0; p < 6; ++p) {
          double s = g[pa[p]][i] * g[pb[p]][j];
          if (pa[p] != pb[p]) s += g[pb[p]][i] * g[pa[p]][j];
          t->stiff[p * nb * nb + i * nb + j] += w * s;
        }
      }
  }
  return MG_OK;
}

// -------------------------------------------------------------------- edges --
// Unique edges bucketed by their smaller node id; the bucket lists are filled in
// element x local-edge order, so the first incidence of an edge is its first
// appearance.  LEX numbers edges by (min, max); FIRST by first appearance.
mg_status ensure_edges(mg_mesh* m)
{
  if (m->n_edges >= 0) return MG_OK;
  const int64_t N = m->n_nodes, E = m->n_elem, M = 6 * E;
  std::vector<int64_t> start(N + 1, 0);
  for (int64_t e = 0; e < E; ++e)
    for (int j = 0; j < 6; ++j) {
      int32_t a = m->conn[4 * e + kEdgePts[j][0]], b = m->conn[4 * e + kEdgePts[j][1]];
      start[std::min(a, b) + 1]++;
    }
  for (int64_t i = 0; i < N; ++i) start[i + 1] += start[i];
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  std::vector<int32_t> inc_hi(M);
  std::vector<int64_t> inc_idx(M);
  for (int64_t e = 0; e < E; ++e)
    for (int j = 0; j < 6; ++j) {
      int32_t a = m->conn[4 * e + kEdgePts[j][0]], b = m->conn[4 * e + kEdgePts[j][1]];
      int64_t pos = fill[std::min(a, b)]++;
      inc_hi[pos] = std::max(a, b);
      inc_idx[pos] = 6 * e + j;
    }
  // per bucket: unique his (sorted) and the first incidence of each; a bucket
  // holds any number of edges (a vertex may start hundreds)
  std::vector<int32_t> nuniq(N + 1, 0);
  std::vector<int32_t> local_rank(M);  // rank of the incidence's edge within its bucket
#pragma omp parallel
  {
    std::vector<int32_t> his;
#pragma omp for schedule(dynamic, 4096)
    for (int64_t v = 0; v < N; ++v) {
      his.assign(inc_hi.begin() + start[v], inc_hi.begin() + start[v + 1]);
      std::sort(his.begin(), his.end());
      his.erase(std::unique(his.begin(), his.end()), his.end());
      nuniq[v + 1] = (int32_t)his.size();
      for (int64_t t = start[v]; t < start[v + 1]; ++t)
        local_rank[t] = (int32_t)(std::lower_bound(his.begin(), his.end(), inc_hi[t]) - his.begin());
    }
  }
  for (int64_t v = 0; v < N; ++v) nuniq[v + 1] += nuniq[v];
  const int64_t nE = nuniq[N];
  // lex gid of every incidence, and first incidence of every edge
  std::vector<int32_t> lex_of_inc(M);
  std::vector<int64_t> first(nE, INT64_MAX);
  for (int64_t v = 0; v < N; ++v)
    for (int64_t t = start[v]; t < start[v + 1]; ++t) {
      int32_t g = nuniq[v] + local_rank[t];
      lex_of_inc[inc_idx[t]] = g;
      if (inc_idx[t] < first[g]) first[g] = inc_idx[t];
    }
  std::vector<int32_t> gid_of_lex(nE);
  if (m->edge_rule == MG_EDGES_LEX) {
    for (int64_t g = 0; g < nE; ++g) gid_of_lex[g] = (int32_t)g;
  } else {
    // first appearance: order edges by their first incidence (unique values < 6E)
    std::vector<int32_t> by_first(M, -1);
    for (int64_t g = 0; g < nE; ++g) by_first[first[g]] = (int32_t)g;
    int32_t k = 0;
    for (int64_t t = 0; t < M; ++t)
      if (by_first[t] >= 0) gid_of_lex[by_first[t]] = k++;
  }
  m->elem_edge.resize(M);
  for (int64_t t = 0; t < M; ++t) m->elem_edge[t] = gid_of_lex[lex_of_inc[t]];
  m->edge_nodes.resize(2 * nE);
  for (int64_t g = 0; g < nE; ++g) {
    const int64_t e = first[g] / 6;
    const int j = (int)(first[g] % 6);
    const int32_t gid = gid_of_lex[g];
    m->edge_nodes[2 * gid] = m->conn[4 * e + kEdgePts[j][0]];
    m->edge_nodes[2 * gid + 1] = m->conn[4 * e + kEdgePts[j][1]];
  }
  m->n_edges = nE;
  return MG_OK;
}

mg_status check_device(int want, const char* what)
{
  int dev = -1;
  MG_CUDA(cudaGetDevice(&dev));
  if (dev != want)
    return set_error(MG_ERR_INVALID_ARG, std::string(what) + " was uploaded to device " + std::to_string(want) +
                                             ", but device " + std::to_string(dev) + " is current");
  return MG_OK;
}

mg_status mesh_device(mg_mesh* m)
{
  if (m->on_device) return check_device(m->device, "the mesh");
  std::lock_guard<std::mutex> lock(m->upload_mu);
  if (m->on_device) return check_device(m->device, "the mesh");
  MG_CUDA(cudaGetDevice(&m->device));
  const int64_t N = m->n_nodes, E = m->n_elem;
  std::vector<double4_32a> x64(N);
  std::vector<float4> rec(2 * N);
  std::vector<float> loz(N);
#pragma omp parallel for
  for (int64_t i = 0; i < N; ++i) {
    double c[3] = {m->xyz[3 * i], m->xyz[3 * i + 1], m->xyz[3 * i + 2]};
    float h[3], md[3], l[3];
    for (int k = 0; k < 3; ++k) {  // each remainder is exact in double
      h[k] = (float)c[k];
      const double r1 = c[k] - (double)h[k];
      md[k] = (float)r1;
      l[k] = (float)(r1 - (double)md[k]);
    }
    x64[i] = make_double4_32a(c[0], c[1], c[2], 0.0);
    rec[2 * i] = make_float4(h[0], h[1], h[2], md[0]);
    rec[2 * i + 1] = make_float4(md[1], md[2], l[0], l[1]);
    loz[i] = l[2];
  }
  MG_CUDA(cudaMalloc(&m->d_xyz, sizeof(double4_32a) * std::max<int64_t>(N, 1)));
  MG_CUDA(cudaMalloc(&m->d_node_rec, 2 * sizeof(float4) * std::max<int64_t>(N, 1)));
  MG_CUDA(cudaMalloc(&m->d_lo_z, sizeof(float) * std::max<int64_t>(N, 1)));
  MG_CUDA(cudaMalloc(&m->d_conn, sizeof(int4) * std::max<int64_t>(E, 1)));
  MG_CUDA(cudaMalloc(&m->d_dofs, sizeof(int32_t) * std::max<int64_t>(E * m->nb, 1)));
  MG_CUDA(cudaMemcpy(m->d_xyz, x64.data(), sizeof(double4_32a) * N, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(m->d_node_rec, rec.data(), 2 * sizeof(float4) * N, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(m->d_lo_z, loz.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
  MG_CUDA(cudaMemcpy(m->d_conn, m->conn.data(), sizeof(int4) * E, cudaMemcpyHostToDevice));
  if (m->order == 1)  // P1 dofs = the connectivity, already on the device
    MG_CUDA(cudaMemcpy(m->d_dofs, m->d_conn, sizeof(int32_t) * E * 4, cudaMemcpyDeviceToDevice));
  else
    MG_CUDA(cudaMemcpy(m->d_dofs, m->dofs.data(), sizeof(int32_t) * E * m->nb, cudaMemcpyHostToDevice));
  m->on_device = true;
  return MG_OK;
}

static void free_mesh(mg_mesh* m)
{
  if (!m) return;
  cudaFree(m->d_xyz);
  cudaFree(m->d_node_rec);
  cudaFree(m->d_lo_z);
  cudaFree(m->d_conn);
  cudaFree(m->d_dofs);
  delete m;
}

static mg_status finish_mesh(mg_mesh* m)
{
  const int64_t N = m->n_nodes, E = m->n_elem;
  // node ids in range, distinct within a tet (checked in parallel; the first
  // offending element is then found in order, for the message)
  auto elem_ok = [&](int64_t e) {
    const int32_t* c = &m->conn[4 * e];
    for (int s = 0; s < 4; ++s) {
      if (c[s] < 0 || c[s] >= N) return false;
      for (int t = 0; t < s; ++t)
        if (c[s] == c[t]) return false;
    }
    return true;
  };
  int ids_bad = 0;
#pragma omp parallel for reduction(max : ids_bad)
  for (int64_t e = 0; e < E; ++e)
    if (!elem_ok(e)) ids_bad = 1;
  if (ids_bad)
    for (int64_t e = 0; e < E; ++e) {
      const int32_t* c = &m->conn[4 * e];
      for (int s = 0; s < 4; ++s) {
        if (c[s] < 0 || c[s] >= N)
          return set_error(MG_ERR_BAD_MESH, "element " + std::to_string(e) + " has node id " +
                                                std::to_string(c[s]) + " outside [0, n_nodes)");
        for (int t = 0; t < s; ++t)
          if (c[s] == c[t])
            return set_error(MG_ERR_BAD_MESH, "element " + std::to_string(e) + " repeats a node");
      }
    }
  // finite coordinates (a NaN would also slip through the minimum below)
  int nonfinite = 0;
#pragma omp parallel for reduction(max : nonfinite)
  for (int64_t i = 0; i < 3 * N; ++i)
    if (!std::isfinite(m->xyz[i])) nonfinite = 1;
  if (nonfinite)
    for (int64_t i = 0; i < 3 * N; ++i)
      if (!std::isfinite(m->xyz[i]))
        return set_error(MG_ERR_BAD_MESH, "node " + std::to_string(i / 3) + " has a non-finite coordinate");
  // Jacobian check: the map is affine, so detJ is the same at every vertex.
  double mn = INFINITY;
  int64_t bad = -1;
  int any_bad = 0;
#pragma omp parallel for reduction(min : mn) reduction(max : any_bad)
  for (int64_t e = 0; e < E; ++e) {
    const int32_t* c = &m->conn[4 * e];
    double J[3][3];
    for (int k = 0; k < 3; ++k)
      for (int r = 0; r < 3; ++r) J[r][k] = m->xyz[3 * (int64_t)c[k + 1] + r] - m->xyz[3 * (int64_t)c[0] + r];
    double d = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (d < mn) mn = d;
    if (!(d > 0.0)) any_bad = 1;
  }
  m->min_det = E > 0 ? mn : 0.0;
  if (E > 0 && (any_bad || !(mn > 0.0))) {
    for (int64_t e = 0; e < E && bad < 0; ++e) {
      const int32_t* c = &m->conn[4 * e];
      double J[3][3];
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) J[r][k] = m->xyz[3 * (int64_t)c[k + 1] + r] - m->xyz[3 * (int64_t)c[0] + r];
      double d = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                 J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      if (!(d > 0.0)) bad = e;
    }
    return set_error(MG_ERR_BAD_MESH, "element " + std::to_string(bad) +
                                          " has detJ <= 0 (min detJ " + std::to_string(mn) + ")");
  }
  // dof map
  m->nb = nbasis(m->order);
  if (m->order == 2)
    MG_TRY(m->edges_on_device ? build_edges_device(m, (cudaStream_t)m->edge_stream) : ensure_edges(m));
  m->ndof = m->order == 1 ? N : N + m->n_edges;
  if (m->order == 2) {  // P1: the dofs are the vertices (mesh_dofs reads conn)
    m->dofs.resize(E * m->nb);
#pragma omp parallel for
    for (int64_t e = 0; e < E; ++e) {
      for (int v = 0; v < 4; ++v) m->dofs[m->nb * e + v] = m->conn[4 * e + v];
      for (int j = 0; j < 6; ++j) m->dofs[m->nb * e + 4 + j] = (int32_t)(N + m->elem_edge[6 * e + j]);
    }
  }
  if (m->ndof >= INT32_MAX) return set_error(MG_ERR_SIZE, "more than 2^31-1 dofs");
  return MG_OK;
}

}  // namespace mg

using namespace mg;

// dst = src[0 .. n), copied in chunks over the host threads
template <typename T>
static void parallel_copy(std::vector<T>& dst, const T* src, int64_t n)
{
  dst.resize(n);
  const int64_t chunk = 1 << 20;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < (n + chunk - 1) / chunk; ++c)
    std::memcpy(dst.data() + c * chunk, src + c * chunk, sizeof(T) * (size_t)std::min(chunk, n - c * chunk));
}

extern "C" {

static mg_status create_mesh(mg_mesh** out, int64_t n_nodes, const double* h_xyz, int64_t n_elements,
                             const int32_t* h_conn, int32_t order, int32_t edge_rule, bool on_device, void* stream)
{
  if (!out || n_nodes < 0 || n_elements < 0 || (n_nodes > 0 && !h_xyz) ||
      (n_elements > 0 && !h_conn))
    return set_error(MG_ERR_INVALID_ARG, "mg_mesh_create: null or negative argument");
  if (order != 1 && order != 2) return set_error(MG_ERR_INVALID_ARG, "order must be 1 or 2");
  if (edge_rule != MG_EDGES_LEX && edge_rule != MG_EDGES_FIRST)
    return set_error(MG_ERR_INVALID_ARG, "edge_rule must be MG_EDGES_LEX or MG_EDGES_FIRST");
  if (n_nodes >= INT32_MAX || n_elements >= (int64_t)INT32_MAX / 16)
    return set_error(MG_ERR_SIZE, "mesh larger than the int32 index range");
  *out = nullptr;
  mg_mesh* m = new mg_mesh();
  m->order = order;
  m->edge_rule = edge_rule;
  m->edges_on_device = on_device;
  m->edge_stream = stream;
  m->nb = nbasis(order);
  m->n_nodes = n_nodes;
  m->n_elem = n_elements;
  parallel_copy(m->xyz, h_xyz, 3 * n_nodes);
  parallel_copy(m->conn, h_conn, 4 * n_elements);
  mg_status s = finish_mesh(m);
  if (s != MG_OK) {
    free_mesh(m);
    return s;
  }
  *out = m;
  return MG_OK;
}

mg_status mg_mesh_create(mg_mesh** out, int64_t n_nodes, const double* h_xyz, int64_t n_elements,
                         const int32_t* h_conn, int32_t order, int32_t edge_rule)
{
  NvtxRange nvtx_range("mg_mesh_create");
  return create_mesh(out, n_nodes, h_xyz, n_elements, h_conn, order, edge_rule, false, nullptr);
}

mg_status mg_mesh_create_device(mg_mesh** out, int64_t n_nodes, const double* h_xyz, int64_t n_elements,
                                const int32_t* h_conn, int32_t order, int32_t edge_rule, void* stream)
{
  NvtxRange nvtx_range("mg_mesh_create_device");
  return create_mesh(out, n_nodes, h_xyz, n_elements, h_conn, order, edge_rule, true, stream);
}

mg_status mg_mesh_load_gmsh(mg_mesh** out, const char* path, int32_t order, int32_t edge_rule)
{
  NvtxRange nvtx_range("mg_mesh_load_gmsh");
  if (!out || !path) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_load_gmsh: null argument");
  std::ifstream f(path);
  if (!f) return set_error(MG_ERR_IO, std::string("cannot open ") + path);
  std::string line;
  std::vector<double> xyz;
  std::vector<int32_t> conn, tris, tri_geo;
  int64_t n_nodes = -1;
  while (std::getline(f, line)) {
    if (line.find("$Nodes") != std::string::npos) {
      if (!std::getline(f, line)) return set_error(MG_ERR_IO, "truncated $Nodes");
      n_nodes = std::stoll(line);
      xyz.resize(3 * n_nodes);
      for (int64_t i = 0; i < n_nodes; ++i) {
        if (!std::getline(f, line)) return set_error(MG_ERR_IO, "truncated $Nodes");
        std::istringstream is(line);
        double label, x, y, z;  // the file's node label is ignored: gid = line order
        if (!(is >> label >> x >> y >> z)) return set_error(MG_ERR_IO, "bad node line: " + line);
        xyz[3 * i] = x; xyz[3 * i + 1] = y; xyz[3 * i + 2] = z;
      }
    } else if (line.find("$Elements") != std::string::npos) {
      if (!std::getline(f, line)) return set_error(MG_ERR_IO, "truncated $Elements");
      const int64_t n = std::stoll(line);
      for (int64_t i = 0; i < n; ++i) {
        if (!std::getline(f, line)) return set_error(MG_ERR_IO, "truncated $Elements");
        std::istringstream is(line);
        std::vector<int64_t> v;
        int64_t t;
        while (is >> t) v.push_back(t);
        if (v.size() < 3) return set_error(MG_ERR_IO, "bad element line: " + line);
        if (v[1] == 2) {  // boundary triangle: kept with its geoId (2nd tag) for the multipliers
          const int64_t nt = v[2];
          if ((nt != 2 && nt != 3) || (int64_t)v.size() != 3 + nt + 3)
            return set_error(MG_ERR_IO, "triangle with unsupported tag count: " + line);
          for (int k = 0; k < 3; ++k) tris.push_back((int32_t)(v[3 + nt + k] - 1));
          tri_geo.push_back((int32_t)v[4]);
          continue;
        }
        if (v[1] != 4) continue;  // only tetrahedra feed the volume operators
        const int64_t ntags = v[2];
        if ((ntags != 2 && ntags != 3) || (int64_t)v.size() != 3 + ntags + 4)
          return set_error(MG_ERR_IO, "tetrahedron with unsupported tag count: " + line);
        for (int k = 0; k < 4; ++k) conn.push_back((int32_t)(v[3 + ntags + k] - 1));
      }
    }
  }
  if (n_nodes < 0) return set_error(MG_ERR_IO, "no $Nodes section");
  for (const int32_t t : tris)
    if (t < 0 || t >= n_nodes) return set_error(MG_ERR_BAD_MESH, "triangle node id out of range");
  MG_TRY(mg_mesh_create(out, n_nodes, xyz.data(), (int64_t)conn.size() / 4, conn.data(), order, edge_rule));
  (*out)->tri_nodes.swap(tris);
  (*out)->tri_geo.swap(tri_geo);
  return MG_OK;
}

mg_status mg_mesh_export_triangles(const mg_mesh* m, int64_t* n_tris, int32_t* h_tris, int32_t* h_geo_ids)
{
  if (!m) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_export_triangles: null mesh");
  const int64_t n = (int64_t)m->tri_geo.size();
  if (n_tris) *n_tris = n;
  if (h_tris && n) std::memcpy(h_tris, m->tri_nodes.data(), sizeof(int32_t) * 3 * n);
  if (h_geo_ids && n) std::memcpy(h_geo_ids, m->tri_geo.data(), sizeof(int32_t) * n);
  return MG_OK;
}

mg_status mg_mesh_destroy(mg_mesh* mesh)
{
  free_mesh(mesh);
  return MG_OK;
}

mg_status mg_mesh_get_info(const mg_mesh* m, mg_mesh_info* info)
{
  if (!m || !info) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_get_info: null argument");
  info->n_nodes = m->n_nodes;
  info->n_elements = m->n_elem;
  info->n_edges = m->n_edges;
  info->ndof = m->ndof;
  info->order = m->order;
  info->edge_rule = m->edge_rule;
  info->min_det = m->min_det;
  return MG_OK;
}

mg_status mg_mesh_export_dofs(const mg_mesh* m, int32_t* h_elem_dofs)
{
  if (!m || !h_elem_dofs) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_export_dofs: null argument");
  std::memcpy(h_elem_dofs, mesh_dofs(m), sizeof(int32_t) * (size_t)(m->n_elem * m->nb));
  return MG_OK;
}

mg_status mg_mesh_export_edges(const mg_mesh* mc, int32_t* h_edge_nodes, int32_t* h_elem_edges)
{
  mg_mesh* m = const_cast<mg_mesh*>(mc);
  if (!m) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_export_edges: null mesh");
  MG_TRY(ensure_edges(m));
  if (h_edge_nodes)
    std::memcpy(h_edge_nodes, m->edge_nodes.data(), sizeof(int32_t) * m->edge_nodes.size());
  if (h_elem_edges)
    std::memcpy(h_elem_edges, m->elem_edge.data(), sizeof(int32_t) * m->elem_edge.size());
  return MG_OK;
}

mg_status mg_mesh_export_geometry(const mg_mesh* m, double* h_xyz, int32_t* h_conn)
{
  if (!m) return set_error(MG_ERR_INVALID_ARG, "mg_mesh_export_geometry: null mesh");
  if (h_xyz) std::memcpy(h_xyz, m->xyz.data(), sizeof(double) * m->xyz.size());
  if (h_conn) std::memcpy(h_conn, m->conn.data(), sizeof(int32_t) * m->conn.size());
  return MG_OK;
}

const char* mg_status_string(mg_status s)
{
  switch (s) {
    case MG_OK: return "MG_OK";
    case MG_ERR_INVALID_ARG: return "MG_ERR_INVALID_ARG";
    case MG_ERR_CUDA: return "MG_ERR_CUDA";
    case MG_ERR_ALLOC: return "MG_ERR_ALLOC";
    case MG_ERR_BAD_MESH: return "MG_ERR_BAD_MESH";
    case MG_ERR_NOT_CONVERGED: return "MG_ERR_NOT_CONVERGED";
    case MG_ERR_UNSUPPORTED: return "MG_ERR_UNSUPPORTED";
    case MG_ERR_IO: return "MG_ERR_IO";
    case MG_ERR_SIZE: return "MG_ERR_SIZE";
    default: return "MG_ERR_UNKNOWN";
  }
}

const char* mg_last_error(void) { return g_last_error.c_str(); }

const char* mg_version(void) { return "morgana-gb300 0.1 (sm_103a)"; }

}  // extern "C"
