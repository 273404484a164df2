// Boundary multipliers (host side): boundary faces, the P1 multiplier numbering,
// the patterns of B = opLA3dA and of the saddle matrix [K B^T; B 0], and the
// index maps the kernels of mg_lagrange.cu gather through.
//
// Reference behaviour restated here (paths relative to the morganaPublic tree):
//  - boundary faces: faces of exactly one tet (connect3d getFaceIsBoundary),
//    visited in element then local-face order (the builder's loop over grid3d,
//    localMatrixLA3d::matrix, src/morganaFiniteElements/localMatrixLA3d.hpp:292-322);
//  - multipliers (fePr2d<1>): the nodes of the boundary triangles, compacted in
//    ascending node id (meshDoctor2d::removeUnusedPoints, meshDoctor2d.hpp:339-500),
//    numbered in that order (dofMapStatic2d.hpp:1166-1380); (fePr2d<0>): one per
//    triangle, in the boundary grid's element order -- the order of the given
//    triangles, whose ids the boundary elements keep (meshInit3d.hpp:400-430);
//  - B: every face inserts its nt x nb block (rows: the face's multipliers,
//    columns: all nb dofs of the tet, zeros kept), duplicates summed in insertion
//    order (traitsMatrixBuilder.hpp:363-441, Epetra_FECrsMatrix::InsertGlobalValues);
//  - saddle: K on the field block, B on (multiplier, field) and B^T on (field,
//    multiplier) (epetraSaddleAssembler::setDiagMatrix / setSymmMatrix).
#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <numeric>

#include <omp.h>
#include <parallel/algorithm>

#include "mg_internal.h"
#include "mg_lagrange.cuh"

namespace mg {

namespace {

constexpr int64_t kInt32Max = 2147483647;

struct Tri {
  int32_t a, b, c;  // ascending
  bool operator<(const Tri& o) const { return a != o.a ? a < o.a : (b != o.b ? b < o.b : c < o.c); }
  bool operator==(const Tri& o) const { return a == o.a && b == o.b && c == o.c; }
};

Tri sorted_tri(int32_t x, int32_t y, int32_t z)
{
  if (x > y) std::swap(x, y);
  if (y > z) std::swap(y, z);
  if (x > y) std::swap(x, y);
  return Tri{x, y, z};
}

// Flags every local face of every tet: 1 = boundary (one tet), 0 = interior
// (two tets).  A face found in three or more tets makes the mesh invalid.
// Faces are bucketed by their lowest node (parallel counts and scatter with
// atomics; the order inside a bucket is then fixed by sorting it by (other two
// nodes, face id)), so the copies of a face meet in one short sorted bucket.
mg_status boundary_flags(const mg_mesh* m, std::vector<uint8_t>* flag)
{
  const int64_t N = m->n_nodes, E = m->n_elem, F = 4 * E;
  const int32_t* conn = m->conn.data();
  auto face_of = [conn](int64_t f) {
    const int32_t* c = conn + 4 * (f >> 2);
    const int lf = (int)(f & 3);
    return sorted_tri(c[face_vertex(lf, 0)], c[face_vertex(lf, 1)], c[face_vertex(lf, 2)]);
  };
  std::vector<int64_t> start(N + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < F; ++f) {
    const int32_t x = face_of(f).a;
#pragma omp atomic
    start[x + 1]++;
  }
  for (int64_t i = 0; i < N; ++i) start[i + 1] += start[i];
  std::vector<int32_t> bucket(F);
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < F; ++f) {
      const int32_t x = face_of(f).a;
      int64_t pos;
#pragma omp atomic capture
      pos = fill[x]++;
      bucket[pos] = (int32_t)f;
    }
  }
  flag->assign(F, 0);
  int bad = 0;
#pragma omp parallel reduction(| : bad)
  {
    struct Face {
      int32_t b, c, id;  // the face's other two nodes (b < c), 4 e + local face
      bool operator<(const Face& o) const { return b != o.b ? b < o.b : (c != o.c ? c < o.c : id < o.id); }
    };
    std::vector<Face> loc;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t x = 0; x < N; ++x) {
      loc.clear();
      for (int64_t k = start[x]; k < start[x + 1]; ++k) {
        const Tri t = face_of(bucket[k]);
        loc.push_back(Face{t.b, t.c, bucket[k]});
      }
      std::sort(loc.begin(), loc.end());
      for (size_t i = 0; i < loc.size();) {
        size_t j = i + 1;
        while (j < loc.size() && loc[j].b == loc[i].b && loc[j].c == loc[i].c) ++j;
        if (j - i == 1) (*flag)[loc[i].id] = 1;
        if (j - i > 2) bad = 1;
        i = j;
      }
    }
  }
  if (bad) return set_error(MG_ERR_BAD_MESH, "mg_lagrange_build: a face is shared by more than two tets");
  return MG_OK;
}

// Edge j of the P2 test basis of local face lf of element e: face vertices
// (j, j + 1 mod 3), as a (min node, max node) key.
uint64_t face_edge_key(const mg_mesh* m, int32_t e, int lf, int j)
{
  const int32_t* c = m->conn.data() + 4 * (int64_t)e;
  const int32_t p = c[face_vertex(lf, j)], q = c[face_vertex(lf, j == 2 ? 0 : j + 1)];
  return (uint64_t)(uint32_t)std::min(p, q) << 32 | (uint32_t)std::max(p, q);
}

// Boundary faces, element then local-face order, kept as ids 4 e + local face;
// with a triangle list, only those faces, and rank[f] = the list position of
// face f (the boundary grid's element order, which numbers P0 multipliers),
// else rank[f] = f.
// all_ids receives every boundary face (the boundary grid, whatever is selected).
mg_status select_faces(const mg_mesh* m, int64_t n_tris, const int32_t* h_tris, std::vector<int32_t>* ids,
                       std::vector<int64_t>* rank, std::vector<int32_t>* all_ids)
{
  const int64_t E = m->n_elem, N = m->n_nodes;
  std::vector<uint8_t> flag;
  MG_TRY(boundary_flags(m, &flag));
  ids->clear();
  for (int64_t k = 0; k < 4 * E; ++k)
    if (flag[k]) ids->push_back((int32_t)k);
  *all_ids = *ids;
  rank->clear();
  if (!h_tris) {
    rank->resize(ids->size());
    std::iota(rank->begin(), rank->end(), (int64_t)0);
    return MG_OK;
  }
  std::vector<std::pair<Tri, int64_t>> want(n_tris);
  for (int64_t t = 0; t < n_tris; ++t) {
    const int32_t* v = h_tris + 3 * t;
    for (int s = 0; s < 3; ++s)
      if (v[s] < 0 || v[s] >= N) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: triangle node id out of range");
    want[t] = {sorted_tri(v[0], v[1], v[2]), t};
  }
  std::sort(want.begin(), want.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  for (int64_t t = 1; t < n_tris; ++t)
    if (want[t].first == want[t - 1].first)
      return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: a triangle is listed twice");
  std::vector<int32_t> kept;
  for (const int32_t id : *ids) {
    const int32_t* c = m->conn.data() + 4 * (int64_t)(id / 4);
    const int lf = id % 4;
    const Tri t = sorted_tri(c[face_vertex(lf, 0)], c[face_vertex(lf, 1)], c[face_vertex(lf, 2)]);
    auto it = std::lower_bound(want.begin(), want.end(), t,
                               [](const std::pair<Tri, int64_t>& x, const Tri& y) { return x.first < y; });
    if (it != want.end() && it->first == t) {
      kept.push_back(id);
      rank->push_back(it->second);
    }
  }
  if ((int64_t)kept.size() != n_tris)
    return set_error(MG_ERR_BAD_MESH, "mg_lagrange_build: a listed triangle is not a boundary face of the mesh");
  ids->swap(kept);
  return MG_OK;
}

// Multipliers: P1 the nodes of the selected faces, ascending (lam_of[node] =
// its multiplier); P2 those, then the faces' edges in the boundary grid's edge
// order -- MG_EDGES_LEX: (min, max) order; MG_EDGES_FIRST: first appearance over
// every boundary face (all_ids, element then local-face order) and its local
// edges (0,1), (1,2), (2,0) in face-vertex order, as connect2d numbers the edges
// of the boundary grid whose triangles connect3d stores in faceToPoint order.
// edge_index = (key, multiplier offset among the edges), sorted by key.  P0: one
// per face, in the order of `rank`.
void number_multipliers(mg_lagrange* lg, const mg_mesh* m, const std::vector<int64_t>& rank,
                        const std::vector<int32_t>& all_ids, std::vector<int32_t>* lam_of,
                        std::vector<std::pair<uint64_t, int64_t>>* edge_index)
{
  const int64_t N = m->n_nodes, nf = lg->n_faces;
  lg->lam_node.clear();
  lg->lam_edge.clear();
  lam_of->clear();
  edge_index->clear();
  if (lg->test_order == 0) {
    lg->lam_node.resize(nf);
    for (int64_t f = 0; f < nf; ++f) lg->lam_node[rank[f]] = (int32_t)f;
    lg->nl = nf;
    return;
  }
  lam_of->assign(N, -1);
  for (int64_t f = 0; f < nf; ++f) {
    const int32_t* c = m->conn.data() + 4 * (int64_t)lg->face_elem[f];
    for (int a = 0; a < 3; ++a) (*lam_of)[c[face_vertex(lg->face_local[f], a)]] = 0;
  }
  for (int64_t i = 0; i < N; ++i)
    if ((*lam_of)[i] == 0) {
      (*lam_of)[i] = (int32_t)lg->lam_node.size();
      lg->lam_node.push_back((int32_t)i);
    }
  lg->n_vertex_lam = (int64_t)lg->lam_node.size();
  if (lg->test_order == 2) {
    std::vector<uint64_t> keys;  // the selected faces' edges
    keys.reserve(3 * nf);
    for (int64_t f = 0; f < nf; ++f)
      for (int j = 0; j < 3; ++j) keys.push_back(face_edge_key(m, lg->face_elem[f], lg->face_local[f], j));
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    if (m->edge_rule == MG_EDGES_FIRST) {
      // rank of first appearance over the whole boundary grid
      std::vector<std::pair<uint64_t, int64_t>> first;  // (key, first position)
      first.reserve(3 * all_ids.size());
      for (size_t q = 0; q < all_ids.size(); ++q)
        for (int j = 0; j < 3; ++j)
          first.push_back({face_edge_key(m, all_ids[q] / 4, all_ids[q] % 4, j), (int64_t)(3 * q + j)});
      std::sort(first.begin(), first.end());  // by key, then position: the first of each key leads
      auto pos_of = [&first](uint64_t k) {
        return std::lower_bound(first.begin(), first.end(), std::make_pair(k, (int64_t)-1))->second;
      };
      std::sort(keys.begin(), keys.end(), [&](uint64_t x, uint64_t y) { return pos_of(x) < pos_of(y); });
    }
    for (size_t i = 0; i < keys.size(); ++i) {
      lg->lam_node.push_back(-1);
      lg->lam_edge.push_back((int32_t)(keys[i] >> 32));
      lg->lam_edge.push_back((int32_t)(keys[i] & 0xffffffffu));
      edge_index->push_back({keys[i], (int64_t)i});
    }
    std::sort(edge_index->begin(), edge_index->end());
  }
  lg->nl = (int64_t)lg->lam_node.size();
}

// B: (row, column) of every face-matrix entry, sorted by (row, column, source);
// sources are generated ascending, so each entry's list is in insertion order.
void build_b(mg_lagrange* lg, const mg_mesh* m, const std::vector<int64_t>& rank, const std::vector<int32_t>& lam_of,
             const std::vector<std::pair<uint64_t, int64_t>>& edge_index)
{
  const int nb = lg->nb, nt = lg->nt;
  const int64_t nf = lg->n_faces, nl = lg->nl;
  struct Pair {
    uint64_t key;  // row << 32 | column
    int32_t src;   // (f * nt + a) * nb + i
    bool operator<(const Pair& o) const { return key != o.key ? key < o.key : src < o.src; }
  };
  std::vector<Pair> pairs(nf * nt * nb);
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < nf; ++f) {
    const int64_t e = lg->face_elem[f];
    const int32_t* c = m->conn.data() + 4 * e;
    for (int a = 0; a < nt; ++a) {
      uint64_t row;
      if (lg->test_order == 0) {
        row = (uint64_t)rank[f];
      } else if (a < 3) {
        row = (uint64_t)lam_of[c[face_vertex(lg->face_local[f], a)]];
      } else {  // P2 edge function of face edge a - 3
        const uint64_t key = face_edge_key(m, (int32_t)e, lg->face_local[f], a - 3);
        row = (uint64_t)(lg->n_vertex_lam +
                         std::lower_bound(edge_index.begin(), edge_index.end(), std::make_pair(key, (int64_t)-1))
                             ->second);
      }
      for (int i = 0; i < nb; ++i) {
        const int64_t s = (f * nt + a) * nb + i;
        pairs[s] = Pair{row << 32 | (uint64_t)(uint32_t)mesh_dofs(m)[e * nb + i], (int32_t)s};
      }
    }
  }
  __gnu_parallel::sort(pairs.begin(), pairs.end());
  lg->b_rowptr.assign(nl + 1, 0);
  lg->b_colind.clear();
  lg->b_src_ptr.clear();
  lg->b_src.resize(pairs.size());
  for (size_t k = 0; k < pairs.size(); ++k) {
    if (k == 0 || pairs[k].key != pairs[k - 1].key) {
      lg->b_src_ptr.push_back((int32_t)k);
      lg->b_colind.push_back((int32_t)(pairs[k].key & 0xffffffffu));
      lg->b_rowptr[(pairs[k].key >> 32) + 1]++;
    }
    lg->b_src[k] = pairs[k].src;
  }
  lg->b_src_ptr.push_back((int32_t)pairs.size());
  for (int64_t l = 0; l < nl; ++l) lg->b_rowptr[l + 1] += lg->b_rowptr[l];
  lg->nnz_b = (int64_t)lg->b_colind.size();
}

// B^T B (setMTM): every pair of entries (k1, k2) of a multiplier row l couples
// columns (i, j); entry (i, j) sums B[k1] B[k2] over its rows l in ascending
// order.  Structural pattern: zeros kept.  Returns its CSR (ndof rows).
mg_status build_mtm(mg_lagrange* lg, std::vector<int32_t>* m_rowptr, std::vector<int32_t>* m_colind)
{
  const int64_t nl = lg->nl, nd = lg->ndof;
  struct Prod {
    uint64_t key;  // i << 32 | j
    int32_t l, k1, k2;
    bool operator<(const Prod& o) const { return key != o.key ? key < o.key : l < o.l; }
  };
  std::vector<int64_t> off(nl + 1, 0);
  for (int64_t l = 0; l < nl; ++l) {
    const int64_t len = lg->b_rowptr[l + 1] - lg->b_rowptr[l];
    off[l + 1] = off[l] + len * len;
  }
  if (off[nl] > kInt32Max) return set_error(MG_ERR_SIZE, "mg_lagrange_build: B^T B has more than 2^31 - 1 products");
  std::vector<Prod> prods(off[nl]);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t l = 0; l < nl; ++l) {
    int64_t o = off[l];
    for (int32_t k1 = lg->b_rowptr[l]; k1 < lg->b_rowptr[l + 1]; ++k1)
      for (int32_t k2 = lg->b_rowptr[l]; k2 < lg->b_rowptr[l + 1]; ++k2)
        prods[o++] = Prod{(uint64_t)(uint32_t)lg->b_colind[k1] << 32 | (uint32_t)lg->b_colind[k2], (int32_t)l, k1, k2};
  }
  __gnu_parallel::sort(prods.begin(), prods.end());
  m_rowptr->assign(nd + 1, 0);
  m_colind->clear();
  lg->m_pair_ptr.clear();
  lg->m_pairs.resize(prods.size());
  for (size_t k = 0; k < prods.size(); ++k) {
    if (k == 0 || prods[k].key != prods[k - 1].key) {
      lg->m_pair_ptr.push_back((int32_t)k);
      m_colind->push_back((int32_t)(prods[k].key & 0xffffffffu));
      (*m_rowptr)[(prods[k].key >> 32) + 1]++;
    }
    lg->m_pairs[k] = make_int2(prods[k].k1, prods[k].k2);
  }
  lg->m_pair_ptr.push_back((int32_t)prods.size());
  for (int64_t r = 0; r < nd; ++r) (*m_rowptr)[r + 1] += (*m_rowptr)[r];
  lg->nnz_m = (int64_t)m_colind->size();
  return MG_OK;
}

// B B^T (setMMT): every pair of entries (k1, k2) of a field column c couples
// multiplier rows (l1, l2); entry (l1, l2) sums B[k1] B[k2] over its columns c
// in ascending order.  Structural pattern: zeros kept.  Returns its CSR
// (n_multipliers rows, columns = multiplier indices).
mg_status build_mmt(mg_lagrange* lg, std::vector<int32_t>* p_rowptr, std::vector<int32_t>* p_colind)
{
  const int64_t nl = lg->nl, nd = lg->ndof, nzb = lg->nnz_b;
  // B's entries by column, rows ascending within a column (a counting transpose)
  std::vector<int64_t> cstart(nd + 1, 0);
  for (int64_t k = 0; k < nzb; ++k) cstart[lg->b_colind[k] + 1]++;
  for (int64_t c = 0; c < nd; ++c) cstart[c + 1] += cstart[c];
  std::vector<int32_t> by_col(nzb), row_of(nzb);
  {
    std::vector<int64_t> fill(cstart.begin(), cstart.end() - 1);
    for (int64_t l = 0; l < nl; ++l)
      for (int32_t k = lg->b_rowptr[l]; k < lg->b_rowptr[l + 1]; ++k) {
        by_col[fill[lg->b_colind[k]]++] = k;
        row_of[k] = (int32_t)l;
      }
  }
  struct Prod {
    uint64_t key;  // l1 << 32 | l2
    int32_t c, k1, k2;
    bool operator<(const Prod& o) const { return key != o.key ? key < o.key : c < o.c; }
  };
  std::vector<int64_t> off(nd + 1, 0);
  for (int64_t c = 0; c < nd; ++c) {
    const int64_t len = cstart[c + 1] - cstart[c];
    off[c + 1] = off[c] + len * len;
  }
  if (off[nd] > kInt32Max) return set_error(MG_ERR_SIZE, "mg_lagrange_build: B B^T has more than 2^31 - 1 products");
  std::vector<Prod> prods(off[nd]);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < nd; ++c) {
    int64_t o = off[c];
    for (int64_t a = cstart[c]; a < cstart[c + 1]; ++a)
      for (int64_t b = cstart[c]; b < cstart[c + 1]; ++b) {
        const int32_t k1 = by_col[a], k2 = by_col[b];
        prods[o++] = Prod{(uint64_t)(uint32_t)row_of[k1] << 32 | (uint32_t)row_of[k2], (int32_t)c, k1, k2};
      }
  }
  __gnu_parallel::sort(prods.begin(), prods.end());
  p_rowptr->assign(nl + 1, 0);
  p_colind->clear();
  lg->p_pair_ptr.clear();
  lg->p_pairs.resize(prods.size());
  for (size_t k = 0; k < prods.size(); ++k) {
    if (k == 0 || prods[k].key != prods[k - 1].key) {
      lg->p_pair_ptr.push_back((int32_t)k);
      p_colind->push_back((int32_t)(prods[k].key & 0xffffffffu));
      (*p_rowptr)[(prods[k].key >> 32) + 1]++;
    }
    lg->p_pairs[k] = make_int2(prods[k].k1, prods[k].k2);
  }
  lg->p_pair_ptr.push_back((int32_t)prods.size());
  for (int64_t l = 0; l < nl; ++l) (*p_rowptr)[l + 1] += (*p_rowptr)[l];
  lg->nnz_p = (int64_t)p_colind->size();
  return MG_OK;
}

// Saddle: rows r < nd hold the union of K's and (setMTM) B^T B's columns, then
// B^T's (columns nd + l, ascending l); rows nd + l hold B's row l (columns <
// nd), then the union of the diagonal (if requested) and (setMMT) B B^T's
// columns (nd + l2).  Fills s_rowptr / s_colind, the source map s_src, each
// field row's diagonal entry s_diag and the B^T B / B B^T slots m_slot, p_slot.
mg_status build_saddle(mg_lagrange* lg, const std::vector<int32_t>& m_rowptr, const std::vector<int32_t>& m_colind,
                       const std::vector<int32_t>& p_rowptr, const std::vector<int32_t>& p_colind)
{
  const mg_plan* p = lg->plan;
  const int64_t nd = lg->ndof, nl = lg->nl;
  const bool mtm = lg->mtm;
  // K row r and B^T B row r merged by column: calls f(column, K entry or -1, B^T B entry or -1)
  auto merge = [&](int64_t r, auto&& f) {
    int32_t a = p->rowptr[r], b = mtm ? m_rowptr[r] : 0;
    const int32_t a1 = p->rowptr[r + 1], b1 = mtm ? m_rowptr[r + 1] : 0;
    while (a < a1 || b < b1) {
      if (b >= b1 || (a < a1 && p->colind[a] < m_colind[b])) {
        f(p->colind[a], a, -1);
        ++a;
      } else if (a >= a1 || m_colind[b] < p->colind[a]) {
        f(m_colind[b], -1, b);
        ++b;
      } else {
        f(p->colind[a], a, b);
        ++a, ++b;
      }
    }
  };
  // multiplier row l's trailing part: the diagonal (lam_diag) merged with B B^T
  // row l: calls g(multiplier column, is diagonal, B B^T entry or -1)
  auto merge_lam = [&](int64_t l, auto&& g) {
    int32_t b = lg->mmt ? p_rowptr[l] : 0;
    const int32_t b1 = lg->mmt ? p_rowptr[l + 1] : 0;
    bool diag = lg->lam_diag;
    while (diag || b < b1) {
      if (diag && (b >= b1 || (int64_t)p_colind[b] > l)) {
        g((int32_t)l, true, -1);
        diag = false;
      } else if (diag && (int64_t)p_colind[b] == l) {
        g((int32_t)l, true, b);
        diag = false;
        ++b;
      } else {
        g(p_colind[b], false, b);
        ++b;
      }
    }
  };
  std::vector<int32_t> tcnt(nd + 1, 0);
  for (int64_t k = 0; k < lg->nnz_b; ++k) tcnt[lg->b_colind[k] + 1]++;
  for (int64_t r = 0; r < nd; ++r) tcnt[r + 1] += tcnt[r];
  std::vector<int64_t> srp(nd + nl + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < nd; ++r) {
    int64_t n = 0;
    merge(r, [&n](int32_t, int32_t, int32_t) { ++n; });
    srp[r + 1] = n + (tcnt[r + 1] - tcnt[r]);
  }
  for (int64_t r = 0; r < nd; ++r) srp[r + 1] += srp[r];
  for (int64_t l = 0; l < nl; ++l) {
    int64_t n = 0;
    merge_lam(l, [&n](int32_t, bool, int32_t) { ++n; });
    srp[nd + l + 1] = srp[nd + l] + (lg->b_rowptr[l + 1] - lg->b_rowptr[l]) + n;
  }
  const int64_t ns = srp[nd + nl];
  if (ns > kInt32Max || nd + nl > kInt32Max)
    return set_error(MG_ERR_SIZE, "mg_lagrange_build: the saddle matrix has more than 2^31 - 1 entries");
  lg->s_rowptr.assign(srp.begin(), srp.end());
  lg->nnz_s = ns;
  lg->s_colind.resize(ns);
  lg->s_src.resize(ns);
  lg->s_diag.assign(nd, -1);
  lg->m_slot.assign(lg->nnz_m, 0);
  lg->p_slot.assign(lg->nnz_p, 0);
  std::vector<int32_t> tfill(nd);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < nd; ++r) {  // K and B^T B part
    int32_t s = lg->s_rowptr[r];
    merge(r, [&](int32_t col, int32_t ka, int32_t mb) {
      lg->s_colind[s] = col;
      lg->s_src[s] = ka >= 0 ? ka : kSrcZero;
      if (mb >= 0) lg->m_slot[mb] = s;
      if (col == (int32_t)r) lg->s_diag[r] = s;
      ++s;
    });
    tfill[r] = s;
  }
  for (int64_t l = 0; l < nl; ++l)  // B^T part: rows visited in ascending l
    for (int32_t k = lg->b_rowptr[l]; k < lg->b_rowptr[l + 1]; ++k) {
      const int32_t s = tfill[lg->b_colind[k]]++;
      lg->s_colind[s] = (int32_t)(nd + l);
      lg->s_src[s] = -(k + 1);
    }
#pragma omp parallel for schedule(static)
  for (int64_t l = 0; l < nl; ++l) {  // B part, then the diagonal and B B^T
    int32_t s = lg->s_rowptr[nd + l];
    for (int32_t k = lg->b_rowptr[l]; k < lg->b_rowptr[l + 1]; ++k, ++s) {
      lg->s_colind[s] = lg->b_colind[k];
      lg->s_src[s] = -(k + 1);
    }
    merge_lam(l, [&](int32_t col, bool diag, int32_t pb) {
      lg->s_colind[s] = (int32_t)(nd + col);
      lg->s_src[s] = diag ? kSrcLamDiag : kSrcZero;  // the diagonal starts at eye_lam
      if (pb >= 0) lg->p_slot[pb] = s;
      ++s;
    });
  }
  return MG_OK;
}

}  // namespace

static mg_status build_lagrange(mg_lagrange* lg, int test_order, int64_t n_tris, const int32_t* h_tris,
                                bool lam_diag, bool mtm, bool mmt)
{
  const mg_mesh* m = lg->plan->mesh;
  lg->order = m->order;
  lg->nb = m->nb;
  lg->ndof = m->ndof;
  lg->test_order = test_order;
  lg->nt = test_order == 2 ? 6 : (test_order == 1 ? 3 : 1);
  lg->lam_diag = lam_diag;
  lg->mtm = mtm;
  lg->mmt = mmt;
  if (4 * m->n_elem > kInt32Max) return set_error(MG_ERR_SIZE, "mg_lagrange_build: more than 2^29 tets");

  std::vector<int32_t> ids, all_ids;
  std::vector<int64_t> rank;
  MG_TRY(select_faces(m, n_tris, h_tris, &ids, &rank, &all_ids));
  const int64_t nf = (int64_t)ids.size();
  if (nf * lg->nt * lg->nb > kInt32Max) return set_error(MG_ERR_SIZE, "mg_lagrange_build: too many boundary faces");
  lg->n_faces = nf;
  lg->face_elem.resize(nf);
  lg->face_local.resize(nf);
  for (int64_t f = 0; f < nf; ++f) {
    lg->face_elem[f] = ids[f] / 4;
    lg->face_local[f] = ids[f] % 4;
  }

  std::vector<int32_t> lam_of;
  std::vector<std::pair<uint64_t, int64_t>> edge_index;
  number_multipliers(lg, m, rank, all_ids, &lam_of, &edge_index);
  build_b(lg, m, rank, lam_of, edge_index);
  std::vector<int32_t> m_rowptr, m_colind, p_rowptr, p_colind;
  if (mtm) MG_TRY(build_mtm(lg, &m_rowptr, &m_colind));
  if (mmt) MG_TRY(build_mmt(lg, &p_rowptr, &p_colind));
  return build_saddle(lg, m_rowptr, m_colind, p_rowptr, p_colind);
}

template <typename T>
static mg_status upload(T** d, const std::vector<T>& h)
{
  MG_CUDA(cudaMalloc(d, sizeof(T) * std::max<size_t>(h.size(), 1)));
  if (!h.empty()) MG_CUDA(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return MG_OK;
}

static void free_device(mg_lagrange* lg)
{
  cudaFree(lg->d_faces);
  cudaFree(lg->d_b_rowptr);
  cudaFree(lg->d_b_colind);
  cudaFree(lg->d_b_src_ptr);
  cudaFree(lg->d_b_src);
  cudaFree(lg->d_s_rowptr);
  cudaFree(lg->d_s_colind);
  cudaFree(lg->d_s_src);
  cudaFree(lg->d_face_mat);
  cudaFree(lg->d_s_diag);
  lg->d_s_diag = nullptr;
  cudaFree(lg->d_m_pair_ptr);
  cudaFree(lg->d_m_pairs);
  cudaFree(lg->d_m_slot);
  lg->d_m_pair_ptr = lg->d_m_slot = nullptr;
  lg->d_m_pairs = nullptr;
  cudaFree(lg->d_p_pair_ptr);
  cudaFree(lg->d_p_pairs);
  cudaFree(lg->d_p_slot);
  lg->d_p_pair_ptr = lg->d_p_slot = nullptr;
  lg->d_p_pairs = nullptr;
  lg->d_faces = nullptr;
  lg->d_b_rowptr = lg->d_b_colind = lg->d_b_src_ptr = lg->d_b_src = nullptr;
  lg->d_s_rowptr = lg->d_s_colind = lg->d_s_src = nullptr;
  lg->d_face_mat = nullptr;
  lg->on_device = false;
}

mg_status lagrange_device(mg_lagrange* lg)
{
  if (lg->on_device) return check_device(lg->plan->mesh->device, "the multiplier handle");
  std::lock_guard<std::mutex> lock(lg->upload_mu);
  if (lg->on_device) return check_device(lg->plan->mesh->device, "the multiplier handle");
  MG_TRY(plan_device(lg->plan));
  std::vector<int2> faces(lg->n_faces);
  for (int64_t f = 0; f < lg->n_faces; ++f) faces[f] = make_int2(lg->face_elem[f], lg->face_local[f]);
  mg_status s = upload(&lg->d_faces, faces);
  if (s == MG_OK) s = upload(&lg->d_b_rowptr, lg->b_rowptr);
  if (s == MG_OK) s = upload(&lg->d_b_colind, lg->b_colind);
  if (s == MG_OK) s = upload(&lg->d_b_src_ptr, lg->b_src_ptr);
  if (s == MG_OK) s = upload(&lg->d_b_src, lg->b_src);
  if (s == MG_OK) s = upload(&lg->d_s_rowptr, lg->s_rowptr);
  if (s == MG_OK) s = upload(&lg->d_s_colind, lg->s_colind);
  if (s == MG_OK) s = upload(&lg->d_s_src, lg->s_src);
  if (s == MG_OK) s = upload(&lg->d_s_diag, lg->s_diag);
  if (s == MG_OK && lg->mtm) s = upload(&lg->d_m_pair_ptr, lg->m_pair_ptr);
  if (s == MG_OK && lg->mtm) s = upload(&lg->d_m_pairs, lg->m_pairs);
  if (s == MG_OK && lg->mtm) s = upload(&lg->d_m_slot, lg->m_slot);
  if (s == MG_OK && lg->mmt) s = upload(&lg->d_p_pair_ptr, lg->p_pair_ptr);
  if (s == MG_OK && lg->mmt) s = upload(&lg->d_p_pairs, lg->p_pairs);
  if (s == MG_OK && lg->mmt) s = upload(&lg->d_p_slot, lg->p_slot);
  if (s == MG_OK) {
    const cudaError_t e =
        cudaMalloc(&lg->d_face_mat, sizeof(double) * std::max<int64_t>(lg->n_faces * lg->nt * lg->nb, 1));
    if (e != cudaSuccess) s = cuda_error(e, "cudaMalloc(face matrices)");
  }
  if (s != MG_OK) {
    free_device(lg);
    return s;
  }
  lg->on_device = true;
  return MG_OK;
}

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_lagrange_build(mg_plan* plan, int32_t test_order, int64_t n_tris, const int32_t* h_tris,
                            int32_t flags, mg_lagrange** out)
{
  NvtxRange nvtx_range("mg_lagrange_build");
  if (!plan || !out) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: null argument");
  if (test_order < 0 || test_order > 2)
    return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: multipliers are P0 (0), P1 (1) or P2 (2)");
  if (flags & ~(MG_SADDLE_LAM_DIAG | MG_SADDLE_MTM | MG_SADDLE_MMT))
    return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: bad flags");
  if (n_tris < 0 || (n_tris > 0 && !h_tris)) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_build: bad triangle list");
  *out = nullptr;
  mg_lagrange* lg = new (std::nothrow) mg_lagrange();
  if (!lg) return set_error(MG_ERR_ALLOC, "mg_lagrange_build: out of host memory");
  lg->plan = plan;
  mg_status s;
  try {
    s = build_lagrange(lg, test_order, n_tris, h_tris, (flags & MG_SADDLE_LAM_DIAG) != 0,
                       (flags & MG_SADDLE_MTM) != 0, (flags & MG_SADDLE_MMT) != 0);
  } catch (const std::bad_alloc&) {
    s = set_error(MG_ERR_ALLOC, "mg_lagrange_build: out of host memory");
  }
  if (s != MG_OK) {
    delete lg;
    return s;
  }
  *out = lg;
  return MG_OK;
}

mg_status mg_lagrange_destroy(mg_lagrange* lg)
{
  if (!lg) return MG_OK;
  free_device(lg);
  delete lg;
  return MG_OK;
}

mg_status mg_lagrange_get_info(const mg_lagrange* lg, mg_lagrange_info* info)
{
  if (!lg || !info) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_get_info: null argument");
  info->n_faces = lg->n_faces;
  info->n_multipliers = lg->nl;
  info->ndof = lg->ndof;
  info->nnz_b = lg->nnz_b;
  info->nnz_saddle = lg->nnz_s;
  info->nnz_mtm = lg->nnz_m;
  info->n_edge_multipliers = (int64_t)lg->lam_edge.size() / 2;
  info->nnz_mmt = lg->nnz_p;
  info->n_mmt_products = (int64_t)lg->p_pairs.size();
  info->n_mtm_products = (int64_t)lg->m_pairs.size();
  return MG_OK;
}

mg_status mg_lagrange_export(const mg_lagrange* lg, int32_t* h_lam_node, int32_t* h_face_elem, int32_t* h_face_local)
{
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_export: null handle");
  if (h_lam_node && lg->nl) std::memcpy(h_lam_node, lg->lam_node.data(), sizeof(int32_t) * lg->nl);
  if (h_face_elem && lg->n_faces) std::memcpy(h_face_elem, lg->face_elem.data(), sizeof(int32_t) * lg->n_faces);
  if (h_face_local && lg->n_faces) std::memcpy(h_face_local, lg->face_local.data(), sizeof(int32_t) * lg->n_faces);
  return MG_OK;
}

mg_status mg_lagrange_pattern(const mg_lagrange* lg, int32_t* h_b_rowptr, int32_t* h_b_colind, int32_t* h_s_rowptr,
                              int32_t* h_s_colind)
{
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_pattern: null handle");
  if (h_b_rowptr) std::memcpy(h_b_rowptr, lg->b_rowptr.data(), sizeof(int32_t) * lg->b_rowptr.size());
  if (h_b_colind && lg->nnz_b) std::memcpy(h_b_colind, lg->b_colind.data(), sizeof(int32_t) * lg->nnz_b);
  if (h_s_rowptr) std::memcpy(h_s_rowptr, lg->s_rowptr.data(), sizeof(int32_t) * lg->s_rowptr.size());
  if (h_s_colind && lg->nnz_s) std::memcpy(h_s_colind, lg->s_colind.data(), sizeof(int32_t) * lg->nnz_s);
  return MG_OK;
}

mg_status mg_lagrange_export_maps(const mg_lagrange* lg, int32_t* h_b_src_ptr, int32_t* h_b_src, int32_t* h_s_src)
{
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_export_maps: null handle");
  if (h_b_src_ptr) std::memcpy(h_b_src_ptr, lg->b_src_ptr.data(), sizeof(int32_t) * lg->b_src_ptr.size());
  if (h_b_src && !lg->b_src.empty()) std::memcpy(h_b_src, lg->b_src.data(), sizeof(int32_t) * lg->b_src.size());
  if (h_s_src && lg->nnz_s) std::memcpy(h_s_src, lg->s_src.data(), sizeof(int32_t) * lg->nnz_s);
  return MG_OK;
}

mg_status mg_lagrange_export_edges(const mg_lagrange* lg, int32_t* h_edge_nodes)
{
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_export_edges: null handle");
  if (h_edge_nodes && !lg->lam_edge.empty())
    std::memcpy(h_edge_nodes, lg->lam_edge.data(), sizeof(int32_t) * lg->lam_edge.size());
  return MG_OK;
}

mg_status mg_lagrange_export_products(const mg_lagrange* lg, int32_t which, int32_t* h_pair_ptr, int32_t* h_pairs,
                                      int32_t* h_slot)
{
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_export_products: null handle");
  if (which != MG_SADDLE_MTM && which != MG_SADDLE_MMT)
    return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_export_products: which is MG_SADDLE_MTM or MG_SADDLE_MMT");
  const bool mt = which == MG_SADDLE_MTM;
  if (!(mt ? lg->mtm : lg->mmt)) return MG_OK;
  const std::vector<int32_t>& ptr = mt ? lg->m_pair_ptr : lg->p_pair_ptr;
  const std::vector<int2>& pairs = mt ? lg->m_pairs : lg->p_pairs;
  const std::vector<int32_t>& slot = mt ? lg->m_slot : lg->p_slot;
  if (h_pair_ptr) std::memcpy(h_pair_ptr, ptr.data(), sizeof(int32_t) * ptr.size());
  if (h_pairs && !pairs.empty()) std::memcpy(h_pairs, pairs.data(), sizeof(int2) * pairs.size());
  if (h_slot && !slot.empty()) std::memcpy(h_slot, slot.data(), sizeof(int32_t) * slot.size());
  return MG_OK;
}

}  // extern "C"
