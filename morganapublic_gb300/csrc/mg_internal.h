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

// --------------------------------------------------------- schedule sizes --
// Threads per assembly CTA; each owns the accumulator slots s with s % kThreads
// equal to its thread index.
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// Accumulator slots (CSR entries of the rows a CTA owns) held in shared memory.
constexpr int kAccMax = 8192;
// Owned rows per block (rows of elements have at least nb >= 4 entries, so only
// dofs outside every element can reach it); the kernel stages one block's row
// metadata in shared memory at once.
constexpr int kRowsMax = kAccMax / 4;
// Chunk-record stages of the assembly kernel: record c + kRecStages is copied
// into the stage of record c, its place read from record c.
constexpr int kRecStages = 4;
// Elements ("items") per chunk: one thread per P1 element, eight per P2 element.
constexpr int kChunkP1 = 256;
constexpr int kChunkP2 = 32;
constexpr int kP2ThreadsPerItem = kThreads / kChunkP2;
// Contributions are applied in pieces: all contributions of a piece belong to one
// accumulator slot; the kernel sums a piece in registers and updates the slot
// once.  A piece is 8 bytes (two 32-bit words, the lower one first) and carries
// piece_srcs(order) sources, each indexing the chunk's element matrices (stored
// symmetric, nb (nb + 1) / 2 unique entries, entry-major):
//   P1  4 sources of 12 bits at bits 0, 12, 24, 36 and the slot (14 bits) at bit 48
//   P2  2 words, each source (13 bits) | slot (14 bits) << 13 (the slot in both)
// Padding sources are the zero source (the entry past the chunk's matrices);
// padding pieces target the dummy slot kAccMax.
constexpr uint32_t kSrcBits = 13, kSlotBits = 14;
constexpr uint32_t kSrcMask = (1u << kSrcBits) - 1, kSlotMask = (1u << kSlotBits) - 1;
constexpr uint32_t kP1SrcBits = 12, kP1SrcMask = (1u << kP1SrcBits) - 1, kP1SlotShift = 48;
inline __host__ __device__ constexpr int piece_srcs(int order) { return order == 1 ? 4 : 2; }
// Stages of contribution words in shared memory: the words of chunk q go to
// stage q % kWordStages, so copies run up to that many chunks ahead.
constexpr int kWordStages = 4;

// Values of precision `prec` are doubles (MG_F64, MG_F64_NATIVE) or floats (MG_F32).
inline bool prec_valid(int prec) { return prec == MG_F64 || prec == MG_F32 || prec == MG_F64_NATIVE; }
inline bool prec_is_f64(int prec) { return prec == MG_F64 || prec == MG_F64_NATIVE; }

inline int nbasis(int order) { return order == 1 ? 4 : 10; }
inline int nunique(int order) { return order == 1 ? 10 : 55; }
inline int chunk_items(int order) { return order == 1 ? kChunkP1 : kChunkP2; }
// Index of the symmetric pair (i, j), i <= j, in row-major upper-triangle order.
inline __host__ __device__ int sym_index(int i, int j, int nb)
{
  if (i > j) { const int t = i; i = j; j = t; }
  return i * nb - i * (i - 1) / 2 + (j - i);
}

// One CTA of the assembly kernel: a set of owned rows plus every element that
// touches one of them.
struct BlockDesc {
  int32_t item_begin;   // into items[]
  int32_t item_count;
  int32_t chunk_begin;  // into chunk_ptr[] (in chunks)
  int32_t nchunks;
  int32_t row_begin;    // into rows[] / row_acc[]
  int32_t row_count;
  int32_t acc_used;     // accumulator slots in use
  int32_t word_begin32; // first contribution word of the block / 32
};

// Head of a chunk record.  The plan lays out, per chunk, one contiguous record
// the kernel stages into shared memory with a single bulk copy:
//   ChunkDesc (64 B) | the items' element Morton ranks (4 B x n4; the kernel
//   reads each element's coefficient from a copy in that order)
//   | local vertex indices (4 x 2 B x n4)
//   | vertex coordinates relative to the chunk's first vertex, split exactly
//     r = hi + mid + lo: float4 (hi.xyz, mid.x) x nn | float4 (mid.yz, lo.xy) x nn
//     | float lo.z x nn
// n4 = the chunk's items rounded up to 4, nn = n_nodes (a multiple of 4), so
// every part starts on a 16-byte boundary.  Element matrices depend on edge
// vectors only, so the origin is not needed.
struct ChunkDesc {
  int64_t word_begin;         // first contribution word of the chunk (multiple of 32)
  int32_t warp_off[kWarps + 1];  // per-warp offsets relative to word_begin; [kWarps] = chunk size
  int32_t n_nodes;            // distinct vertices of the chunk's elements (multiple of 4)
  int32_t next_off16;         // record of chunk + kRecStages of the same block: offset / 16
  int32_t next_bytes;         //   and size (0 when the block has no such chunk); the
                              //   kernel takes record places from the chunk table
  int32_t pad[2];
};
static_assert(sizeof(ChunkDesc) == 64, "ChunkDesc must stay 64 bytes");

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

namespace mg { struct HostSchedule; }

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
  std::vector<int32_t> dofs;        // n_elem * nb
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
  // assembly schedule
  int32_t nblocks = 0;
  int64_t n_items = 0, n_item_slots = 0, n_chunks = 0, n_entries = 0, n_contrib = 0;
  mg::BlockDesc* d_blocks = nullptr;
  unsigned char* d_chunk_data = nullptr;  // chunk records (see ChunkDesc), 16-byte aligned
  int2* d_chunk_rec = nullptr;            // (offset / 16, bytes) of each chunk record
  int64_t* d_chunk_wb = nullptr;          // first contribution word of each chunk (n_chunks + 1)
  int32_t max_rec_bytes = 0;
  int32_t max_chunk_nodes = 0;
  int2* d_row_meta = nullptr;  // owned rows, schedule order: (accumulator base, CSR start - base)
  int32_t* d_sched_rows = nullptr;  // device-built schedules: the owned rows (for the schedule export)
  int32_t* d_elem_order = nullptr;  // elements along a Morton curve of their centroids
  double* d_coeff_m = nullptr;      // the coefficient of the current assembly in that order (n_elem)
  int32_t* d_dofs_morton = nullptr; // their dofs (nb each) in that order
  uint32_t* d_entries = nullptr;   // contribution words
  uint32_t* d_counters = nullptr;   // [0] work counter, [1] exit counter, [2] device error, [3] detail
  int64_t max_chunk_entries = 0;
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
  mg::HostSchedule* host_schedule = nullptr;  // until uploaded
  uint32_t wait_limit = MG_WAIT_LIMIT_DEFAULT;  // polls of an assembly pipeline wait (mg_plan_set_wait_limit)
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
// Host copy of the assembly schedule, kept until the plan is first used on the GPU.
struct HostSchedule {
  std::vector<BlockDesc> blocks;
  std::vector<int32_t> items, rows, row_acc;
  std::vector<int64_t> chunk_ptr;
  std::vector<uint32_t> entries;
  int64_t n_contrib = 0;
  int64_t max_chunk_entries = 0;
  // per chunk: its distinct vertices (first-appearance order, padded to 4) and,
  // per item, the local indices of the item's four vertices
  std::vector<int32_t> chunk_node_begin, chunk_n_nodes;
  std::vector<int32_t> chunk_nodes;  // global node ids
  std::vector<uint16_t> item_lconn;  // 4 per item slot
  std::vector<int32_t> elem_order;   // all elements along a Morton curve of their centroids
  int32_t max_chunk_nodes = 0;
};
// MG_OK when `want` is the calling thread's current device, else
// MG_ERR_INVALID_ARG naming both: a handle's device arrays are only valid on
// the device they were uploaded to
mg_status check_device(int want, const char* what);
mg_status mesh_device(mg_mesh* m);  // uploads the mesh on first GPU use
mg_status plan_device(mg_plan* p);  // uploads mesh + plan on first GPU use
mg_status plan_tables(mg_plan* p, int quad, const RefTables** t, const double** d_tab);
mg_status plan_work(mg_plan* p, size_t bytes, void** ptr);
mg_status plan_rhs_map(mg_plan* p);  // the load-vector slot map (once per plan)
int64_t schedule_block_count(int64_t wtot, int64_t wmax, int64_t sms);  // blocks of the schedule (mg_plan.cpp)
// CSR pattern on the GPU (mg_pattern.cu); keep_device: its device arrays become
// the plan's d_rowptr / d_colind
mg_status build_pattern_device(mg_plan* p, cudaStream_t st, bool keep_device);
// the assembly schedule on the GPU from the plan's device pattern (mg_schedule.cu):
// the same arrays as the host build, uploaded state included (on_device)
mg_status build_schedule_device(mg_plan* p, cudaStream_t st);
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
