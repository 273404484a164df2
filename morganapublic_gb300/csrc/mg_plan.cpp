// CSR pattern and plan state (host side).
//
// Pattern: the union of element couplings with sorted columns and explicit
// zeros kept -- the matrix traitsMatrixBuilder::buildEpetraCrs leaves behind
// after Epetra_FECrsMatrix::GlobalAssemble
// (src/morganaFiniteElements/traitsMatrixBuilder.hpp:363-544 in morganaPublic).
//
// Element order: the assembly visits the elements along a Morton curve of their
// centroids, so that neighbouring threads read neighbouring vertices and a block
// of consecutive elements covers a compact region.  The assembly's map from
// element-matrix entries to CSR entries -- the block map (P1) or the slot map
// (P2) -- is built on the GPU from the uploaded pattern (mg_schedule.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

#include <omp.h>
#include <parallel/algorithm>

#include "mg_internal.h"

namespace mg {

static uint64_t spread21(uint64_t v)
{
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

static mg_status build_pattern(mg_plan* p)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = m->ndof;
  const int32_t* dofs = mesh_dofs(m);
  // dof -> incident elements (the order inside a row does not matter: the
  // row's columns are de-duplicated and sorted below)
  std::vector<int64_t> start(nd + 1, 0);
#pragma omp parallel for
  for (int64_t k = 0; k < E * nb; ++k) {
#pragma omp atomic
    start[dofs[k] + 1]++;
  }
  for (int64_t r = 0; r < nd; ++r) start[r + 1] += start[r];
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  std::vector<int32_t> inc(E * nb);
#pragma omp parallel for
  for (int64_t k = 0; k < E * nb; ++k) {
    int64_t slot;
#pragma omp atomic capture
    slot = fill[dofs[k]]++;
    inc[slot] = (int32_t)(k / nb);
  }
  // one pass over the rows: the union of the incident elements' dofs,
  // de-duplicated with a per-thread stamp array (so only the ~15 unique columns
  // of a P1 row are sorted), kept per thread and copied after the prefix sum
  std::vector<int32_t> len(nd, 0);
  const int nth = std::max(1, omp_get_max_threads());
  std::vector<std::vector<int32_t>> cols(nth);
  std::vector<int64_t> chunk_row0(nth + 1, 0);
#pragma omp parallel num_threads(nth)
  {
    const int t = omp_get_thread_num();
    const int64_t r0 = nd * t / nth, r1 = nd * (t + 1) / nth;
    chunk_row0[t] = r0;
    std::vector<int32_t> stamp(nd, -1);
    std::vector<int32_t>& out = cols[t];
    std::vector<int32_t> tmp;
    for (int64_t r = r0; r < r1; ++r) {
      tmp.clear();
      for (int64_t k = start[r]; k < start[r + 1]; ++k)
        for (int i = 0; i < nb; ++i) {
          const int32_t c = dofs[(int64_t)inc[k] * nb + i];
          if (stamp[c] != (int32_t)r) {
            stamp[c] = (int32_t)r;
            tmp.push_back(c);
          }
        }
      std::sort(tmp.begin(), tmp.end());
      len[r] = (int32_t)tmp.size();
      out.insert(out.end(), tmp.begin(), tmp.end());
    }
  }
  p->rowptr.assign(nd + 1, 0);
  for (int64_t r = 0; r < nd; ++r) {
    int64_t next = (int64_t)p->rowptr[r] + len[r];
    if (next >= INT32_MAX) return set_error(MG_ERR_SIZE, "nnz above 2^31-1");
    p->rowptr[r + 1] = (int32_t)next;
  }
  p->nnz = p->rowptr[nd];
  p->colind.resize(p->nnz);
#pragma omp parallel for num_threads(nth)
  for (int t = 0; t < nth; ++t)
    std::copy(cols[t].begin(), cols[t].end(), p->colind.begin() + p->rowptr[chunk_row0[t]]);
  p->ndof = nd;
  return MG_OK;
}

// Elements along a Morton curve of their centroids (0.25 x_v summed over v in
// order, keys of 21 bits per axis over the nodes' bounding box), ties by element
// id -- the keys and order the device build computes (mg_schedule.cu).
static mg_status build_elem_order(mg_plan* p)
{
  mg_mesh* m = p->mesh;
  const int64_t E = m->n_elem, N = m->n_nodes;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], m->xyz[3 * i + k]);
      hi[k] = std::max(hi[k], m->xyz[3 * i + k]);
    }
  std::vector<std::pair<uint64_t, int32_t>> kv(E);
#pragma omp parallel for
  for (int64_t e = 0; e < E; ++e) {
    double x[3] = {0.0, 0.0, 0.0};
    for (int v = 0; v < 4; ++v)
      for (int k = 0; k < 3; ++k) x[k] += 0.25 * m->xyz[3 * (int64_t)m->conn[4 * e + v] + k];
    uint64_t c = 0;
    for (int k = 0; k < 3; ++k) {
      const double t = hi[k] > lo[k] ? (x[k] - lo[k]) / (hi[k] - lo[k]) : 0.0;
      const uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, t * 2097151.0));
      c |= spread21(q) << k;
    }
    kv[e] = std::make_pair(c, (int32_t)e);
  }
  __gnu_parallel::sort(kv.begin(), kv.end());  // by key, ties by element id
  p->h_elem_order.resize(E);
#pragma omp parallel for
  for (int64_t e = 0; e < E; ++e) p->h_elem_order[e] = kv[e].second;
  return MG_OK;
}

template <typename T>
static mg_status upload(T** dst, const std::vector<T>& src)
{
  MG_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
  if (!src.empty()) MG_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return MG_OK;
}

mg_status plan_device(mg_plan* p)
{
  if (p->on_device) return check_device(p->mesh->device, "the plan");
  std::lock_guard<std::mutex> lock(p->upload_mu);
  if (p->on_device) return check_device(p->mesh->device, "the plan");
  MG_TRY(mesh_device(p->mesh));
  MG_TRY(upload(&p->d_rowptr, p->rowptr));
  MG_TRY(upload(&p->d_colind, p->colind));
  std::vector<int32_t> diag(p->ndof);
  for (int64_t r = 0; r < p->ndof; ++r) {
    const int32_t* c0 = p->colind.data() + p->rowptr[r];
    const int32_t* c1 = p->colind.data() + p->rowptr[r + 1];
    diag[r] = p->rowptr[r] + (int32_t)(std::lower_bound(c0, c1, (int32_t)r) - c0);
  }
  MG_TRY(upload(&p->d_diag, diag));
  {
    // 16-bit column offsets (col - row) when every entry fits: 2 bytes per entry
    // less for the SpMV and CG kernels; the CSR arrays stay the reference's
    bool fits = true;
    std::vector<int16_t> off(p->colind.size());
#pragma omp parallel for reduction(&& : fits)
    for (int64_t r = 0; r < p->ndof; ++r)
      for (int32_t k = p->rowptr[r]; k < p->rowptr[r + 1]; ++k) {
        const int64_t d = (int64_t)p->colind[k] - r;
        if (d < INT16_MIN || d > INT16_MAX) fits = false;
        else off[k] = (int16_t)d;
      }
    if (fits && !off.empty()) MG_TRY(upload(&p->d_coloff, off));
  }
  {
    const int nb = p->mesh->nb;
    const int64_t E = (int64_t)p->h_elem_order.size();
    std::vector<int32_t> dm((size_t)E * nb);
#pragma omp parallel for
    for (int64_t i = 0; i < E; ++i)
      for (int k = 0; k < nb; ++k) dm[i * nb + k] = mesh_dofs(p->mesh)[(int64_t)p->h_elem_order[i] * nb + k];
    MG_TRY(upload(&p->d_elem_order, p->h_elem_order));
    MG_TRY(upload(&p->d_dofs_morton, dm));
  }
  MG_TRY(upload(&p->d_counters, std::vector<uint32_t>(8, 0u)));
  MG_CUDA(cudaMallocHost(&p->h_pinned, 64 * sizeof(double)));
  MG_TRY(build_slot_map(p, cudaStreamLegacy));
  p->on_device = true;
  return MG_OK;
}

static void free_plan(mg_plan* p)
{
  if (!p) return;
  cudaFree(p->d_rowptr);
  cudaFree(p->d_colind);
  cudaFree(p->d_diag);
  cudaFree(p->d_coloff);
  cudaFree(p->d_elem_order);
  cudaFree(p->d_dofs_morton);
  cudaFree(p->d_goff);
  cudaFree(p->d_uslot);
  cudaFree(p->d_umirror);
  cudaFree(p->d_src);
  cudaFree(p->d_em);
  cudaFree(p->d_bgrp);
  cudaFree(p->d_bsrc0);
  cudaFree(p->d_bgoff);
  cudaFree(p->d_bsrc);
  cudaFree(p->d_bout);
  cudaFree(p->d_sgoff);
  cudaFree(p->d_sout);
  cudaFree(p->d_partial);
  cudaFree(p->d_rhs_ptr);
  cudaFree(p->d_rhs_slot);
  cudaFree(p->d_rhs_y);
  cudaFree(p->d_geo_det);
  cudaFree(p->d_geo_cof);
  cudaFree(p->d_counters);
  for (double* t : p->d_tables) cudaFree(t);
  cudaFree(p->d_work);
  cudaFree(p->d_tmp_values);
  cudaFree(p->d_tmp_coeff);
  if (p->h_pinned) cudaFreeHost(p->h_pinned);
  delete p;
}

mg_status plan_tables(mg_plan* p, int quad, const RefTables** t, const double** d_tab)
{
  for (size_t k = 0; k < p->tables.size(); ++k)
    if (p->tables[k].quad == quad) {
      *t = &p->tables[k];
      *d_tab = p->d_tables[k];
      return MG_OK;
    }
  RefTables rt;
  MG_TRY(build_ref_tables(p->mesh->order, quad, &rt));
  // device layout: unique (i <= j, sym_index order) entries, stiff[6][nu] then mass[nu]
  const int nb = rt.nb, nu = nb * (nb + 1) / 2;
  std::vector<double> flat(7 * nu);
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j) {
      const int u = sym_index(i, j, nb);
      for (int q = 0; q < 6; ++q) flat[q * nu + u] = rt.stiff[q * nb * nb + i * nb + j];
      flat[6 * nu + u] = rt.mass[i * nb + j];
    }
  double* d = nullptr;
  MG_CUDA(cudaMalloc(&d, sizeof(double) * flat.size()));
  MG_CUDA(cudaMemcpy(d, flat.data(), sizeof(double) * flat.size(), cudaMemcpyHostToDevice));
  p->tables.push_back(rt);
  p->d_tables.push_back(d);
  *t = &p->tables.back();
  *d_tab = d;
  return MG_OK;
}

// Load-vector map: for each dof (natural order), the element-vector slots
// q = p * nb + l with dofs_morton[q] == dof, ascending -- the fixed order in
// which the gather kernel sums them.  A parallel counting transpose, then each
// dof's short list sorted.
mg_status plan_rhs_map(mg_plan* p)
{
  if (p->d_rhs_ptr) return MG_OK;
  const mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = p->ndof, pairs = E * nb;
  if (pairs >= INT32_MAX) return set_error(MG_ERR_SIZE, "load-vector map above 2^31 element-vector entries");
  if ((int64_t)p->h_elem_order.size() != E) return set_error(MG_ERR_INVALID_ARG, "plan without an element order");
  const int32_t* eo = p->h_elem_order.data();
  const int32_t* dofs = mesh_dofs(m);
  auto dof_of = [&](int64_t q) { return dofs[(int64_t)eo[q / nb] * nb + q % nb]; };
  std::vector<int32_t> ptr(nd + 1, 0), slot(std::max<int64_t>(pairs, 1));
#pragma omp parallel for
  for (int64_t q = 0; q < pairs; ++q) {
    const int32_t d = dof_of(q);
#pragma omp atomic
    ptr[d + 1]++;
  }
  for (int64_t d = 0; d < nd; ++d) ptr[d + 1] += ptr[d];
  std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
#pragma omp parallel for
  for (int64_t q = 0; q < pairs; ++q) {
    const int32_t d = dof_of(q);
    int32_t at;
#pragma omp atomic capture
    at = cur[d]++;
    slot[at] = (int32_t)q;
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t d = 0; d < nd; ++d) std::sort(slot.begin() + ptr[d], slot.begin() + ptr[d + 1]);
  // all three buffers or none (the map counts as built once d_rhs_ptr is set)
  int32_t *d_ptr = nullptr, *d_slot = nullptr;
  double* d_y = nullptr;
  mg_status st = upload(&d_ptr, ptr);
  if (st == MG_OK) st = upload(&d_slot, slot);
  if (st == MG_OK) {
    const cudaError_t e = cudaMalloc(&d_y, sizeof(double) * std::max<int64_t>(pairs, 1));
    if (e != cudaSuccess) st = cuda_error(e, "load-vector buffer");
  }
  if (st != MG_OK) {
    cudaFree(d_ptr);
    cudaFree(d_slot);
    cudaFree(d_y);
    return st;
  }
  p->d_rhs_ptr = d_ptr;
  p->d_rhs_slot = d_slot;
  p->d_rhs_y = d_y;
  return MG_OK;
}

mg_status plan_work(mg_plan* p, size_t bytes, void** ptr)
{
  if (p->work_bytes < bytes) {
    cudaFree(p->d_work);
    p->d_work = nullptr;
    p->work_bytes = 0;
    MG_CUDA(cudaMalloc(&p->d_work, bytes));
    p->work_bytes = bytes;
  }
  *ptr = p->d_work;
  return MG_OK;
}

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_pattern_build(mg_mesh* mesh, mg_plan** out)
{
  NvtxRange nvtx_range("mg_pattern_build");
  if (!mesh || !out) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_build: null argument");
  *out = nullptr;
  mg_plan* p = new mg_plan();
  p->mesh = mesh;
  mg_status s = build_pattern(p);
  if (s == MG_OK) s = build_elem_order(p);
  if (s != MG_OK) {
    free_plan(p);
    return s;
  }
  *out = p;
  return MG_OK;
}

mg_status mg_pattern_build_device(mg_mesh* mesh, mg_plan** out, void* stream)
{
  NvtxRange nvtx_range("mg_pattern_build_device");
  if (!mesh || !out) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_build_device: null argument");
  *out = nullptr;
  mg_plan* p = new mg_plan();
  p->mesh = mesh;
  mg_status s = build_pattern_device(p, (cudaStream_t)stream, true);
  if (s == MG_OK) s = build_plan_device(p, (cudaStream_t)stream);
  if (s != MG_OK) {
    free_plan(p);
    return s;
  }
  *out = p;
  return MG_OK;
}

mg_status mg_plan_destroy(mg_plan* plan)
{
  free_plan(plan);
  return MG_OK;
}

mg_status mg_pattern_info(const mg_plan* p, int64_t* ndof, int64_t* nnz)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_info: null plan");
  if (ndof) *ndof = p->ndof;
  if (nnz) *nnz = p->nnz;
  return MG_OK;
}

mg_status mg_pattern_export(const mg_plan* p, int32_t* h_rowptr, int32_t* h_colind)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_export: null plan");
  if (h_rowptr) std::memcpy(h_rowptr, p->rowptr.data(), sizeof(int32_t) * p->rowptr.size());
  if (h_colind) std::memcpy(h_colind, p->colind.data(), sizeof(int32_t) * p->colind.size());
  return MG_OK;
}

mg_status mg_pattern_device(const mg_plan* pc, const int32_t** d_rowptr, const int32_t** d_colind)
{
  mg_plan* p = const_cast<mg_plan*>(pc);
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_device: null plan");
  MG_TRY(plan_device(p));
  if (d_rowptr) *d_rowptr = p->d_rowptr;
  if (d_colind) *d_colind = p->d_colind;
  return MG_OK;
}

mg_status mg_plan_slot_map_info(mg_plan* p, mg_slot_map_info* info)
{
  if (!p || !info) return set_error(MG_ERR_INVALID_ARG, "mg_plan_slot_map_info: null argument");
  if (uses_block_map(p->mesh->order))
    return set_error(MG_ERR_UNSUPPORTED, "P1 plans assemble through the block map (mg_plan_block_map_info)");
  MG_TRY(plan_device(p));
  info->n_upper = p->n_upper;
  info->n_groups = p->n_groups;
  info->n_diag = p->n_diag;
  info->n_contrib = p->n_slot_contrib;
  info->n_src = p->n_src;
  info->n_elem = p->mesh->n_elem;
  info->nunique = nunique(p->mesh->order);
  info->elem_major = slot_map_aos(p->mesh->order) ? 1 : 0;
  info->rows_per_block = kGatherRowBlock;
  info->reserved = 0;
  return MG_OK;
}

mg_status mg_plan_export_slot_map(mg_plan* p, int32_t* h_elem_order, int32_t* h_goff, int32_t* h_uslot,
                                  int32_t* h_umirror, uint32_t* h_src)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_plan_export_slot_map: null plan");
  if (uses_block_map(p->mesh->order))
    return set_error(MG_ERR_UNSUPPORTED, "P1 plans assemble through the block map (mg_plan_export_block_map)");
  MG_TRY(plan_device(p));
  const int64_t E = p->mesh->n_elem, U = p->n_upper, G = p->n_groups, S = p->n_src;
  if (h_elem_order && E) std::memcpy(h_elem_order, p->h_elem_order.data(), sizeof(int32_t) * E);
  if (h_goff) MG_CUDA(cudaMemcpy(h_goff, p->d_goff, sizeof(int32_t) * (G + 1), cudaMemcpyDeviceToHost));
  if (h_uslot && U) MG_CUDA(cudaMemcpy(h_uslot, p->d_uslot, sizeof(int32_t) * U, cudaMemcpyDeviceToHost));
  if (h_umirror && U) MG_CUDA(cudaMemcpy(h_umirror, p->d_umirror, sizeof(int32_t) * U, cudaMemcpyDeviceToHost));
  if (h_src && S) MG_CUDA(cudaMemcpy(h_src, p->d_src, sizeof(uint32_t) * S, cudaMemcpyDeviceToHost));
  return MG_OK;
}

mg_status mg_plan_block_map_info(mg_plan* p, mg_block_map_info* info)
{
  if (!p || !info) return set_error(MG_ERR_INVALID_ARG, "mg_plan_block_map_info: null argument");
  if (!uses_block_map(p->mesh->order))
    return set_error(MG_ERR_UNSUPPORTED, "P2 plans assemble through the slot map (mg_plan_slot_map_info)");
  MG_TRY(plan_device(p));
  info->n_upper = p->n_upper;
  info->n_contrib = p->n_slot_contrib;
  info->n_blocks = p->n_blocks;
  info->n_groups = p->n_bgroups;
  info->n_src = p->n_bsrc;
  info->n_runs = p->n_runs;
  info->n_shared = p->n_shared;
  info->n_shared_groups = p->n_sgroups;
  info->n_partial = p->n_partial;
  info->n_elem = p->mesh->n_elem;
  info->nunique = nunique(p->mesh->order);
  info->elems_per_block = elems_per_block(p->mesh->order);
  return MG_OK;
}

mg_status mg_plan_export_block_map(mg_plan* p, int32_t* h_elem_order, int32_t* h_bgrp, int32_t* h_goff,
                                   uint16_t* h_src, int32_t* h_out, int32_t* h_sgoff, int32_t* h_sout)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_plan_export_block_map: null plan");
  if (!uses_block_map(p->mesh->order))
    return set_error(MG_ERR_UNSUPPORTED, "P2 plans assemble through the slot map (mg_plan_export_slot_map)");
  MG_TRY(plan_device(p));
  const int64_t E = p->mesh->n_elem, G = p->n_bgroups, G3 = p->n_sgroups;
  if (h_elem_order && E) std::memcpy(h_elem_order, p->h_elem_order.data(), sizeof(int32_t) * E);
  if (h_bgrp) MG_CUDA(cudaMemcpy(h_bgrp, p->d_bgrp, sizeof(int32_t) * (p->n_blocks + 1), cudaMemcpyDeviceToHost));
  if (h_goff) MG_CUDA(cudaMemcpy(h_goff, p->d_bgoff, sizeof(int32_t) * (G + 1), cudaMemcpyDeviceToHost));
  if (h_src && p->n_bsrc)
    MG_CUDA(cudaMemcpy(h_src, p->d_bsrc, sizeof(uint16_t) * p->n_bsrc, cudaMemcpyDeviceToHost));
  if (h_out && G) MG_CUDA(cudaMemcpy(h_out, p->d_bout, sizeof(int2) * 32 * G, cudaMemcpyDeviceToHost));
  if (h_sgoff) MG_CUDA(cudaMemcpy(h_sgoff, p->d_sgoff, sizeof(int32_t) * (G3 + 1), cudaMemcpyDeviceToHost));
  if (h_sout && G3) MG_CUDA(cudaMemcpy(h_sout, p->d_sout, sizeof(int2) * 32 * G3, cudaMemcpyDeviceToHost));
  return MG_OK;
}

mg_status mg_plan_export_elem_order(const mg_plan* p, int32_t* h_elem_order)
{
  if (!p || (!h_elem_order && p->mesh->n_elem > 0))
    return set_error(MG_ERR_INVALID_ARG, "mg_plan_export_elem_order: null argument");
  if (p->mesh->n_elem) std::memcpy(h_elem_order, p->h_elem_order.data(), sizeof(int32_t) * p->mesh->n_elem);
  return MG_OK;
}

}  // extern "C"
