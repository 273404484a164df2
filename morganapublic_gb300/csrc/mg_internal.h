// Internal structures of libmorgana_gpu.so (not part of the C ABI).
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "morgana_gpu.h"

namespace mg {

// ------------------------------------------------------------------ errors --
mg_status set_error(mg_status s, const std::string& msg);
mg_status cuda_error(cudaError_t e, const char* what);

#define MG_CUDA(call)                                          \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) return ::mg::cuda_error(_e, #call); \
  } while (0)

// NVTX range over one C-ABI call (header-only NVTX3: no cost and no library
// dependency unless a profiler is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

#define MG_TRY(call)                  \
  do {                                \
    mg_status _s = (call);            \
    if (_s != MG_OK) return _s;       \
  } while (0)

// Values of precision `prec` are doubles (MG_F64, MG_F64_NATIVE) or floats (MG_F32).
inline bool prec_valid(int prec) { return prec == MG_F64 || prec == MG_F32 || prec == MG_F64_NATIVE; }
inline bool prec_is_f64(int prec) { return prec == MG_F64 || prec == MG_F64_NATIVE; }

inline int nbasis(int order) { return order == 1 ? 4 : 10; }
inline int nunique(int order) { return order == 1 ? 10 : 55; }
// Index of the symmetric pair (i, j), i <= j, in row-major upper-triangle order.
inline __host__ __device__ int sym_index(int i, int j, int nb)
{
  if (i > j) { const int t = i; i = j; j = t; }
  return i * nb - i * (i - 1) / 2 + (j - i);
}

// Reference-element tables for one (order, quadrature) pair, with the quadrature
// weights folded in.  stiff[ab][i*nb+j] = sum_q w_q dphi_i/dxi_a dphi_j/dxi_b for
// the six symmetric pairs ab = 00,11,22,01,02,12 (off-diagonal pairs symmetrised);
// mass[i*nb+j] = sum_q w_q phi_i phi_j.  Index i is the field (column) basis
// function and j the test (row) one, the reference's column-major local layout.
struct RefTables {
  int order = 0, quad = 0, nb = 0, nq = 0;
  std::vector<double> stiff;  // 6 * nb * nb
  std::vector<double> mass;   // nb * nb
  double wsum = 0.0;
};
mg_status build_ref_tables(int order, int quad, RefTables* t);
int quad_rule(int quad, std::vector<double>* Y, std::vector<double>* W);
void basis_values(int order, const double* Y, double* v);
void basis_grads(int order, const double* Y, double* gx, double* gy, double* gz);

}  // namespace mg

// ---------------------------------------------------------------- handles --
struct mg_mesh {
  int order = 1, edge_rule = MG_EDGES_LEX, nb = 4, device = 0;
  bool edges_on_device = false;  // P2 edge enumeration on the GPU (mg_mesh_create_device)
  void* edge_stream = nullptr;
  int64_t n_nodes = 0, n_elem = 0, n_edges = -1, ndof = 0;
  double min_det = 0.0;
  std::vector<double> xyz;          // n_nodes * 3
  std::vector<int32_t> conn;        // n_elem * 4
  std::vector<int32_t> elem_edge;   // n_elem * 6 (when built)
  std::vector<int32_t> edge_nodes;  // n_edges * 2 (when built)
  std::vector<int32_t> dofs;        // n_elem * nb (P2; P1 reads conn: mesh_dofs)
  std::vector<int32_t> tri_nodes;   // Gmsh ingest: boundary triangles (3 node ids each), file order
  std::vector<int32_t> tri_geo;     //   and their geoIds (2nd tag)
  // device copies
  double4_32a* d_xyz = nullptr;      // (x, y, z, 0)
  // x = hi + mid + lo exactly (three floats per coordinate), packed so that
  // one 32-byte sector holds a node's (hi.xyz, mid.xyz, lo.x, lo.y); lo.z apart
  float4* d_node_rec = nullptr;  // 2 float4 per node
  float* d_lo_z = nullptr;
  int4* d_conn = nullptr;        // vertex node ids
  int32_t* d_dofs = nullptr;     // n_elem * nb
  // set once the device copies exist (first GPU use, under upload_mu); `device`
  // is the device they live on
  std::atomic<bool> on_device{false};
  std::mutex upload_mu;
};

struct mg_plan {
  mg_mesh* mesh = nullptr;
  int64_t ndof = 0, nnz = 0;
  std::vector<int32_t> rowptr, colind;
  int32_t* d_rowptr = nullptr;
  int32_t* d_colind = nullptr;
  int32_t* d_diag = nullptr;  // slot of the diagonal entry of each row
  int16_t* d_coloff = nullptr; // col - row of every entry when all fit in 16 bits (else null): SpMV index stream
  int32_t* d_elem_order = nullptr;  // elements along a Morton curve of their centroids
  int32_t* d_dofs_morton = nullptr; // their dofs (nb each) in that order
  uint32_t* d_counters = nullptr;   // [4]: assembly flags (bit 0 NaN / Inf coefficient, bit 1 double-word range)
  // slot map of the two-pass (P2) gather assembly (built with the plan's device
  // state; see build_slot_map): the diagonal and upper CSR entries in groups of 32 (one per
  // warp; per block of kGatherRowBlock rows the diagonal entries first), entry t
  // written to uslot[t] and umirror[t];
  // group g's sources src[goff[g] + 32 j + lane], j < (goff[g+1] - goff[g]) / 32,
  // padded with kPadSource
  int32_t* d_goff = nullptr;        // n_groups + 1
  int32_t* d_uslot = nullptr;       // n_upper
  int32_t* d_umirror = nullptr;     // n_upper
  uint32_t* d_src = nullptr;        // n_src
  int64_t n_upper = 0, n_groups = 0, n_diag = 0, n_slot_contrib = 0, n_src = 0;
  void* d_em = nullptr;             // P2 element matrices, nunique x n_elem entries (up to 8 bytes each)
  // block map of the one-pass P1 assembly (build_block_map): elements in blocks
  // of kElemBlock consecutive Morton positions, one CTA each.  Block b's local
  // entries (the runs of an upper entry's sources that fall in the block, longest
  // first) are the groups bgrp[b] .. bgrp[b+1] of 32 lanes; group g's local sources
  // bsrc[bgoff[g] + 32 j + lane] (16-bit (p - b kElemBlock) nu + u, padded with
  // kElemBlock nu), its outputs bout[32 g + lane]: (CSR entry, mirror) of a
  // complete entry, (-1 - q, 0) for partial sum q of a shared entry, kNoOutput
  // for an empty lane.  Shared entries (sources in several blocks) in groups of
  // 32: partials partial[sgoff[g] + 32 j + lane], j < (sgoff[g+1] - sgoff[g]) / 32
  // in ascending block (zero past a lane's count), written to sout[32 g + lane]
  int32_t* d_bgrp = nullptr;        // n_blocks + 1
  int32_t* d_bsrc0 = nullptr;       // n_blocks + 1: bgoff[bgrp[b]] (block b's first local source)
  int32_t* d_bgoff = nullptr;       // n_bgroups + 1
  uint16_t* d_bsrc = nullptr;       // n_bsrc
  int2* d_bout = nullptr;           // 32 n_bgroups
  int32_t* d_sgoff = nullptr;       // n_sgroups + 1
  int2* d_sout = nullptr;           // 32 n_sgroups
  void* d_partial = nullptr;        // n_partial slots of 8 bytes (zero at padding)
  int64_t n_blocks = 0, n_bgroups = 0, n_bsrc = 0, n_runs = 0, n_shared = 0, n_sgroups = 0, n_partial = 0;
  // load vector (built on the first mg_assemble_rhs): per dof, the slots p * nb + l
  // (p = Morton position of an element touching it, l = the dof's local index)
  // of the element vectors it sums, ascending; and the element-vector buffer
  std::vector<int32_t> h_elem_order;  // host copy of the Morton element order
  int32_t* d_rhs_ptr = nullptr;       // ndof + 1
  int32_t* d_rhs_slot = nullptr;      // n_elem * nb
  double* d_rhs_y = nullptr;          // n_elem * nb
  // element geometry in double-word form (built on the first call that needs it:
  // load vector, adjoint), Morton order p: det[p] and cofactor k of element p at
  // cof[k * n_elem + p] (k = 3 r + c), each (hi, lo) floats
  float2* d_geo_det = nullptr;
  float2* d_geo_cof = nullptr;
  // reference tables, cached per (quad) on the device
  std::vector<mg::RefTables> tables;
  std::vector<double*> d_tables;  // parallel to tables: stiff (6 nb^2) then mass (nb^2)
  // solver work space (allocated on first use)
  void* d_work = nullptr;
  size_t work_bytes = 0;
  double* h_pinned = nullptr;  // small pinned scalars
  // temporary buffers of the host-buffer entry points
  void* d_tmp_values = nullptr;
  size_t tmp_values_bytes = 0;
  double* d_tmp_coeff = nullptr;
  size_t tmp_coeff_bytes = 0;
  std::atomic<bool> on_device{false};  // set once uploaded (under upload_mu), on the mesh's device
  std::mutex upload_mu;
};

// Saddle entry sources other than K and B entries (see mg_lagrange::s_src).
// kSrcZero: a B^T B or B B^T entry outside the K / multiplier-diagonal pattern.
constexpr int32_t kSrcLamDiag = INT32_MIN;
constexpr int32_t kSrcZero = INT32_MIN + 1;

// Boundary multipliers of a plan (opLA3dA) and the saddle pattern [K B^T; B 0].
struct mg_lagrange {
  mg_plan* plan = nullptr;
  int order = 1, nb = 4;
  int test_order = 1, nt = 3;  // multiplier basis: P1 (3 per face), P0 (1) or P2 (6)
  bool lam_diag = false;  // the saddle pattern holds the multiplier block's diagonal
  int64_t ndof = 0, n_faces = 0, nl = 0, nnz_b = 0, nnz_s = 0;
  std::vector<int32_t> face_elem, face_local;  // selected boundary faces, element then local-face order
  std::vector<int32_t> lam_node;  // node (P1/P2 vertex, ascending), face (P0) or -1 (P2 edge) per multiplier
  std::vector<int32_t> lam_edge;  // P2: (min, max) nodes of each edge multiplier, after the vertex ones
  int64_t n_vertex_lam = 0;
  std::vector<int32_t> b_rowptr, b_colind;     // B: nl x ndof
  // per B entry k, the face-matrix entries it sums, b_src[b_src_ptr[k] .. b_src_ptr[k+1]),
  // each (f * nt + a) * nb + i, ascending (the reference's insertion order)
  std::vector<int32_t> b_src_ptr, b_src;
  std::vector<int32_t> s_rowptr, s_colind;     // saddle: (ndof + nl) rows
  // per saddle entry: the K entry it copies (>= 0), -(k + 1) for B entry k,
  // kSrcLamDiag (the multiplier diagonal) or kSrcZero (a B^T B entry outside K)
  std::vector<int32_t> s_src;
  std::vector<int32_t> s_diag;  // saddle entry of each field row's diagonal, or -1
  // B^T B (setMTM): per entry m, the product pairs (k1, k2) of B entries it sums,
  // m_pairs[m_pair_ptr[m] .. m_pair_ptr[m+1]) in ascending multiplier row, and the
  // saddle slot it adds into
  bool mtm = false;
  int64_t nnz_m = 0;
  std::vector<int32_t> m_pair_ptr, m_slot;
  std::vector<int2> m_pairs;
  // B B^T (setMMT), the same way over the multiplier block: entry (l1, l2) sums
  // B[k1] B[k2] over the columns the rows share, ascending column
  bool mmt = false;
  int64_t nnz_p = 0;
  std::vector<int32_t> p_pair_ptr, p_slot;
  std::vector<int2> p_pairs;
  // device copies (uploaded on first GPU use)
  int2* d_faces = nullptr;  // (element, local face)
  int32_t *d_b_rowptr = nullptr, *d_b_colind = nullptr, *d_b_src_ptr = nullptr, *d_b_src = nullptr;
  int32_t *d_s_rowptr = nullptr, *d_s_colind = nullptr, *d_s_src = nullptr;
  double* d_face_mat = nullptr;  // n_faces * nt * nb
  int32_t* d_s_diag = nullptr;
  int32_t *d_m_pair_ptr = nullptr, *d_m_slot = nullptr;
  int2* d_m_pairs = nullptr;
  int32_t *d_p_pair_ptr = nullptr, *d_p_slot = nullptr;
  int2* d_p_pairs = nullptr;
  std::atomic<bool> on_device{false};  // set once uploaded (under upload_mu), on the plan's device
  std::mutex upload_mu;
};

namespace mg {
// The element -> dof table, n_elem x nb: the connectivity itself for P1.
inline const int32_t* mesh_dofs(const mg_mesh* m) { return m->order == 1 ? m->conn.data() : m->dofs.data(); }
// MG_OK when `want` is the calling thread's current device, else
// MG_ERR_INVALID_ARG naming both: a handle's device arrays are only valid on
// the device they were uploaded to
mg_status check_device(int want, const char* what);
mg_status mesh_device(mg_mesh* m);  // uploads the mesh on first GPU use
mg_status plan_device(mg_plan* p);  // uploads mesh + plan on first GPU use
mg_status plan_tables(mg_plan* p, int quad, const RefTables** t, const double** d_tab);
mg_status plan_work(mg_plan* p, size_t bytes, void** ptr);
mg_status plan_rhs_map(mg_plan* p);  // the load-vector slot map (once per plan)
// CSR pattern on the GPU (mg_pattern.cu); keep_device: its device arrays become
// the plan's d_rowptr / d_colind
mg_status build_pattern_device(mg_plan* p, cudaStream_t st, bool keep_device);
// the plan's device state from its device pattern (mg_schedule.cu): the same
// arrays plan_device makes for a host-built plan, the assembly's map included
// (on_device)
mg_status build_plan_device(mg_plan* p, cudaStream_t st);
// the assembly's map from the plan's device pattern and Morton dofs
// (mg_schedule.cu), once per plan: the per-entry source lists, laid out as the
// block map (P1) or the gather's slot map (P2)
mg_status build_slot_map(mg_plan* p, cudaStream_t st);
bool slot_map_aos(int order);  // element-matrix layout: element-major (true) or entry-major
// padding source of the gather layout; the kernel maps it to the zero entry past
// the element matrices
constexpr uint32_t kPadSource = 0xffffffffu;
// rows per block of the gather's order: a block's diagonal entries, then its
// other upper entries (its element matrices stay in L2 across both)
constexpr int kGatherRowBlock = 256;
// the one-pass P1 assembly: elements per block (one CTA) and the empty-lane
// output of its block map
constexpr int kElemBlock = 512;
inline int elems_per_block(int) { return kElemBlock; }
constexpr int32_t kNoOutput = INT32_MIN;
// the assembly of an element order runs through the block map (one pass, P1)
// or the slot map and the element-matrix array (two passes, P2: blocks of P2
// elements small enough for shared memory -- 128 -- measured slower on GB300 at
// 48^3, 0.478 against 0.384 ms in FP64)
inline bool uses_block_map(int order) { return order == 1; }
// the block map from the per-entry source lists of the slot map (P1 layout,
// p nu + u, ascending p): see mg_plan::d_bgrp
mg_status build_block_map(mg_plan* p, int64_t U, const int32_t* useg, const int32_t* uslot, const int32_t* umirror,
                          const uint32_t* src, cudaStream_t st);
mg_status build_edges_device(mg_mesh* m, cudaStream_t st);    // edges on the GPU (mg_pattern.cu)
mg_status ensure_edges(mg_mesh* m);
mg_status launch_assemble(mg_plan* p, int op, const double* d_coeff, double c, int quad, int prec,
                          void* d_values, cudaStream_t st);
mg_status launch_spmv(mg_plan* p, int prec, const void* vals, const void* x, void* y, cudaStream_t st);
// y = A x for any CSR matrix of `rows` rows (FP64 values and vectors)
mg_status launch_spmv_csr(int64_t rows, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                          const double* vals, const double* x, double* y, cudaStream_t st);
mg_status lagrange_device(mg_lagrange* lg);  // uploads the multiplier tables on first GPU use
}  // namespace mg
