// The assembly schedule built on the GPU: the same arrays as the host build
// (mg_plan.cpp, build_schedule and the upload in plan_device), bit for bit, from
// the device-resident CSR pattern.  The host rules are chosen so that every
// step is a sort, a scan or a per-chunk computation:
//   1. dofs along a Morton curve of their positions (vertex / edge midpoint):
//      64-bit keys, radix-sorted with the dof id (ties by id);
//   2. blocks cut by the prefix sum of the row weights max(len, 4) in that
//      order (schedule_block_count);
//   3. each block's rows ascending, accumulator bases by a scan;
//   4. elements along a Morton curve of their centroids; items = (block, element)
//      for every block an element touches, sorted by block, then Morton rank;
//   5. per chunk (one CTA each): the distinct vertices in first-appearance order,
//      the contribution list sorted by slot (item order inside), segments
//      ranked longest first and dealt in snake order, 8-byte pieces laid out
//      [piece][lane] per warp; then the chunk record and its words.
// Setup-only library calls: CUB radix sorts and scans.
#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "mg_internal.h"

namespace mg {

namespace {

constexpr int kSchedThreads = 256;
constexpr int kMaxRefs = 4 * kChunkP1;       // vertex references of a chunk (P1: 1024, P2: 128)
constexpr int kMaxContrib = kChunkP1 * 16;   // contribution candidates of a chunk (P1: 4096, P2: 3200)

__device__ __forceinline__ uint64_t spread21(uint64_t v)
{
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

struct Box {
  double lo[3], hi[3];
};

// Morton key of a point, as the host computes it (FP64, no contraction possible:
// a difference, a quotient and one product)
__device__ __forceinline__ uint64_t morton(const double x[3], const Box& bx)
{
  uint64_t c = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double t = bx.hi[k] > bx.lo[k] ? __ddiv_rn(__dsub_rn(x[k], bx.lo[k]), __dsub_rn(bx.hi[k], bx.lo[k])) : 0.0;
    const uint64_t q = (uint64_t)fmin(2097151.0, fmax(0.0, __dmul_rn(t, 2097151.0)));
    c |= spread21(q) << k;
  }
  return c;
}

__global__ void k_dof_keys(int64_t nd, int64_t n_nodes, const double4_32a* __restrict__ xyz,
                           const int32_t* __restrict__ edge_nodes, Box bx, uint64_t* __restrict__ keys,
                           int32_t* __restrict__ ids)
{
  const int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= nd) return;
  double x[3];
  if (d < n_nodes) {
    const double4_32a p = xyz[d];
    x[0] = p.x, x[1] = p.y, x[2] = p.z;
  } else {
    const double4_32a a = xyz[edge_nodes[2 * (d - n_nodes)]], b = xyz[edge_nodes[2 * (d - n_nodes) + 1]];
    x[0] = __dmul_rn(0.5, __dadd_rn(a.x, b.x));
    x[1] = __dmul_rn(0.5, __dadd_rn(a.y, b.y));
    x[2] = __dmul_rn(0.5, __dadd_rn(a.z, b.z));
  }
  keys[d] = morton(x, bx);
  ids[d] = (int32_t)d;
}

// centroid as the host forms it: 0.25 x_v summed over v = 0..3 in order
__global__ void k_elem_keys(int64_t E, const int4* __restrict__ conn, const double4_32a* __restrict__ xyz, Box bx,
                            uint64_t* __restrict__ keys, int32_t* __restrict__ ids)
{
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int4 c = conn[e];
  const int v[4] = {c.x, c.y, c.z, c.w};
  double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const double4_32a p = xyz[v[s]];
    x[0] = __dadd_rn(x[0], __dmul_rn(0.25, p.x));
    x[1] = __dadd_rn(x[1], __dmul_rn(0.25, p.y));
    x[2] = __dadd_rn(x[2], __dmul_rn(0.25, p.z));
  }
  keys[e] = morton(x, bx);
  ids[e] = (int32_t)e;
}

// row weight max(len, 4) in Morton order
__global__ void k_weights(int64_t nd, const int32_t* __restrict__ order, const int32_t* __restrict__ rowptr,
                          int64_t* __restrict__ w)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nd) return;
  const int32_t r = order[t];
  w[t] = max(rowptr[r + 1] - rowptr[r], 4);
}

// raw block floor(W_t nbk / W) of Morton position t, and a flag where it changes
__global__ void k_block_flags(int64_t nd, const int64_t* __restrict__ wex, int64_t wtot, int64_t nbk,
                              int32_t* __restrict__ flag)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nd) return;
  const int64_t b = wex[t] * nbk / wtot;
  flag[t] = (t == 0 || b != wex[t - 1] * nbk / wtot) ? 1 : 0;
}

// block of Morton position t (inclusive scan of the flags - 1); block starts;
// per dof its block; the (block, dof) keys of the owned-row sort
__global__ void k_blocks_of(int64_t nd, const int32_t* __restrict__ order, const int32_t* __restrict__ incl,
                            int32_t* __restrict__ bstart, int32_t* __restrict__ block_of_rank,
                            int32_t* __restrict__ block_of, uint64_t* __restrict__ rowkeys)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nd) return;
  const int32_t b = incl[t] - 1;
  if (t == 0 || incl[t - 1] != incl[t]) bstart[b] = (int32_t)t;
  block_of_rank[t] = b;
  block_of[order[t]] = b;
  rowkeys[t] = ((uint64_t)(uint32_t)b << 32) | (uint32_t)order[t];
}

__global__ void k_row_lens(int64_t nd, const uint64_t* __restrict__ rowkeys, const int32_t* __restrict__ rowptr,
                           int32_t* __restrict__ rows, int32_t* __restrict__ lens)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nd) return;
  const int32_t r = (int32_t)(uint32_t)rowkeys[k];
  rows[k] = r;
  lens[k] = rowptr[r + 1] - rowptr[r];
}

// accumulator base of each owned row (within its block) and per dof
__global__ void k_row_acc(int64_t nd, const int32_t* __restrict__ rows, const int32_t* __restrict__ accex,
                          const int32_t* __restrict__ bstart, const int32_t* __restrict__ block_of_rank,
                          int32_t* __restrict__ row_acc, int32_t* __restrict__ row_acc_of)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nd) return;
  const int32_t a = accex[k] - accex[bstart[block_of_rank[k]]];
  row_acc[k] = a;
  row_acc_of[rows[k]] = a;
}

__global__ void k_rank_of(int64_t E, const int32_t* __restrict__ elem_order, int32_t* __restrict__ rank)
{
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < E) rank[elem_order[p]] = (int32_t)p;
}

// distinct blocks of an element's dofs, first-occurrence order
__device__ __forceinline__ int elem_blocks(int64_t e, int nb, const int32_t* __restrict__ dofs,
                                           const int32_t* __restrict__ block_of, int32_t* out)
{
  int n = 0;
  for (int i = 0; i < nb; ++i) {
    const int32_t b = block_of[dofs[e * nb + i]];
    bool seen = false;
    for (int u = 0; u < n; ++u) seen |= (out[u] == b);
    if (!seen) out[n++] = b;
  }
  return n;
}

__global__ void k_item_counts(int64_t E, int nb, const int32_t* __restrict__ dofs, const int32_t* __restrict__ block_of,
                              int32_t* __restrict__ cnt)
{
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  int32_t bs[10];
  cnt[e] = elem_blocks(e, nb, dofs, block_of, bs);
}

__global__ void k_item_keys(int64_t E, int nb, const int32_t* __restrict__ dofs, const int32_t* __restrict__ block_of,
                            const int64_t* __restrict__ off, const int32_t* __restrict__ rank,
                            uint64_t* __restrict__ keys, int32_t* __restrict__ bcount)
{
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  int32_t bs[10];
  const int n = elem_blocks(e, nb, dofs, block_of, bs);
  for (int u = 0; u < n; ++u) {
    keys[off[e] + u] = ((uint64_t)(uint32_t)bs[u] << 32) | (uint32_t)rank[e];
    atomicAdd(&bcount[bs[u]], 1);  // integer counts: the same for any order
  }
}

// the sorted items into each block's padded list
__global__ void k_items_place(int64_t n, const uint64_t* __restrict__ keys, const int32_t* __restrict__ elem_order,
                              const int64_t* __restrict__ cnt_ex, const int64_t* __restrict__ item_begin,
                              int32_t* __restrict__ items)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t b = (int32_t)(keys[k] >> 32);
  items[item_begin[b] + (k - cnt_ex[b])] = elem_order[(uint32_t)keys[k]];
}

// per block: its chunks (owning block, index in the block)
__global__ void k_chunk_owner(int32_t nbk, const int32_t* __restrict__ chunk_begin, const int32_t* __restrict__ nchunks,
                              int32_t* __restrict__ cblk, int32_t* __restrict__ cpos)
{
  const int32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbk) return;
  for (int32_t c = 0; c < nchunks[b]; ++c) {
    cblk[chunk_begin[b] + c] = b;
    cpos[chunk_begin[b] + c] = c;
  }
}

// ------------------------------------------------------- per-chunk work --
// Bitonic sort of n (a power of two) keys in shared memory by the CTA.
template <typename K>
__device__ void cta_sort(K* a, int n)
{
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const K x = a[i], y = a[ixj];
          if ((x > y) == up) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
}

__device__ __forceinline__ int pow2_at_least(int n)
{
  int p = 32;
  while (p < n) p <<= 1;
  return p;
}

// Exclusive scan of n ints in shared memory (in place) by the CTA; returns the total.
__device__ int cta_scan(int* a, int n, int* tmp /* blockDim.x + 1 */)
{
  const int T = blockDim.x, tid = threadIdx.x;
  const int per = (n + T - 1) / T;
  const int i0 = min(n, tid * per), i1 = min(n, i0 + per);
  int s = 0;
  for (int i = i0; i < i1; ++i) s += a[i];
  tmp[tid] = s;
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int t = 0; t < T; ++t) {
      const int v = tmp[t];
      tmp[t] = run;
      run += v;
    }
    tmp[T] = run;
  }
  __syncthreads();
  int run = tmp[tid];
  for (int i = i0; i < i1; ++i) {
    const int v = a[i];
    a[i] = run;
    run += v;
  }
  __syncthreads();
  const int total = tmp[T];
  __syncthreads();
  return total;
}

struct ChunkArgs {
  int order, nb, CI, nu;
  const int32_t* items;        // padded per-block item lists
  const int32_t* rank;         // Morton rank of each element
  const int32_t* item_begin;   // per block
  const int32_t* item_count;   // per block
  const int32_t* nchunks;      // per block
  const int32_t* cblk;         // per chunk
  const int32_t* cpos;
  const int4* conn;
  const int32_t* dofs;
  const int32_t* block_of;     // per dof
  const int32_t* row_acc_of;   // per dof
  const int32_t* rowptr;
  const int32_t* colind;
  const double4_32a* xyz;
  // outputs / inputs of the passes
  int32_t* n_nodes;            // per chunk (pass 1)
  int64_t* words;              // per chunk (pass 1)
  int64_t* contrib;            // per chunk (pass 1)
  const int64_t* word_begin;   // per chunk (pass 2)
  const int64_t* rec_off;      // per chunk (pass 2), bytes
  unsigned char* records;      // pass 2
  uint32_t* entries;           // pass 2
};

struct ChunkSmem {
  uint64_t refs[kMaxRefs];      // (node << 32 | position) of the chunk's vertex references, sorted
  uint32_t ckey[kMaxContrib];   // (slot << 12 | candidate) of its contributions, sorted
  uint32_t skey[kMaxContrib];   // ((512 - len) << 13 | segment), sorted: the longest-first ranking
  int scan[kMaxContrib];        // segment starts
  int first[kMaxRefs];          // per position: its local index if it is a node's first reference
  int node_of[kMaxRefs];        // node of each local vertex (padded with the first)
  uint16_t local_of[kMaxRefs];  // per position: the local index of its node
  int tmp[kSchedThreads + 1];
  int warp_k[kWarps], warp_off[kWarps + 1];
  int n_contrib;
};

// The chunk's vertices in first-appearance order: local_of[p] for reference
// p = 4 it + v and node_of[l] for l < nn (padded to a multiple of 4 with the
// first vertex); returns nn.
__device__ int chunk_vertices(const ChunkArgs& A, ChunkSmem& S, const int32_t* it_ids, int n_items)
{
  const int nref = 4 * n_items, np = pow2_at_least(nref);
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    uint64_t k = ~0ull;
    if (p < nref) {
      const int4 c = A.conn[it_ids[p >> 2]];
      const int v = p & 3;
      const int node = v == 0 ? c.x : (v == 1 ? c.y : (v == 2 ? c.z : c.w));
      k = ((uint64_t)(uint32_t)node << 32) | (uint32_t)p;
    }
    S.refs[p] = k;
    if (p < nref) S.first[p] = 0;
  }
  __syncthreads();
  cta_sort(S.refs, np);
  // a node's first reference heads its run (the sort is by node, then position)
  for (int i = threadIdx.x; i < nref; i += blockDim.x)
    if (i == 0 || (S.refs[i] >> 32) != (S.refs[i - 1] >> 32)) S.first[(uint32_t)S.refs[i]] = 1;
  __syncthreads();
  const int distinct = cta_scan(S.first, nref, S.tmp);  // first[head position] = local index
  for (int i = threadIdx.x; i < nref; i += blockDim.x) {
    int h = i;
    while (h > 0 && (S.refs[h] >> 32) == (S.refs[h - 1] >> 32)) --h;
    const int l = S.first[(uint32_t)S.refs[h]];
    S.local_of[(uint32_t)S.refs[i]] = (uint16_t)l;
    if (h == i) S.node_of[l] = (int)(S.refs[i] >> 32);
  }
  __syncthreads();
  const int nn = (distinct + 3) & ~3;
  for (int l = distinct + threadIdx.x; l < nn; l += blockDim.x) S.node_of[l] = S.node_of[0];
  __syncthreads();
  return nn;
}

__device__ __forceinline__ int sym_idx(int i, int j, int nb)
{
  if (i > j) { const int t = i; i = j; j = t; }
  return i * nb - i * (i - 1) / 2 + (j - i);
}

// The chunk's contributions sorted by slot (S.ckey; item, field, test order
// inside a slot), its segments' starts (S.scan) and their longest-first ranking
// (S.skey); returns the segment count.
__device__ int chunk_segments(const ChunkArgs& A, ChunkSmem& S, const int32_t* it_ids, int n_items, int32_t b)
{
  const int nb = A.nb, nb2 = nb * nb, ncand = n_items * nb2;
  if (threadIdx.x == 0) S.n_contrib = 0;
  __syncthreads();
  for (int cand = threadIdx.x; cand < ncand; cand += blockDim.x) {
    const int it = cand / nb2, i = (cand / nb) % nb, j = cand % nb;
    const int64_t e = it_ids[it];
    const int32_t row = A.dofs[e * nb + j];
    if (A.block_of[row] != b) continue;
    const int32_t col = A.dofs[e * nb + i];
    int lo = A.rowptr[row], hi = A.rowptr[row + 1];
    while (lo < hi) {  // lower_bound of col in the row's sorted columns
      const int mid = (lo + hi) >> 1;
      if (A.colind[mid] < col) lo = mid + 1;
      else hi = mid;
    }
    const uint32_t slot = (uint32_t)(A.row_acc_of[row] + (lo - A.rowptr[row]));
    S.ckey[atomicAdd(&S.n_contrib, 1)] = (slot << 12) | (uint32_t)cand;  // keys unique: order irrelevant
  }
  __syncthreads();
  const int nc = S.n_contrib, npc = pow2_at_least(nc);
  for (int i = nc + threadIdx.x; i < npc; i += blockDim.x) S.ckey[i] = 0xffffffffu;
  __syncthreads();
  cta_sort(S.ckey, npc);
  for (int i = threadIdx.x; i < nc; i += blockDim.x)
    S.scan[i] = (i == 0 || (S.ckey[i] >> 12) != (S.ckey[i - 1] >> 12)) ? 1 : 0;
  __syncthreads();
  const int nseg = cta_scan(S.scan, nc, S.tmp);  // scan[head] = its segment's index
  for (int i = threadIdx.x; i < nc; i += blockDim.x)
    if (i == 0 || (S.ckey[i] >> 12) != (S.ckey[i - 1] >> 12)) S.skey[S.scan[i]] = (uint32_t)i;
  __syncthreads();
  for (int s = threadIdx.x; s < nseg; s += blockDim.x) S.scan[s] = (int)S.skey[s];  // segment starts
  __syncthreads();
  const int nps = pow2_at_least(nseg);
  for (int s = threadIdx.x; s < nps; s += blockDim.x) {
    uint32_t k = 0xffffffffu;
    if (s < nseg) {
      const int len = (s + 1 < nseg ? S.scan[s + 1] : nc) - S.scan[s];
      k = ((uint32_t)(512 - len) << 13) | (uint32_t)s;
    }
    S.skey[s] = k;
  }
  __syncthreads();
  cta_sort(S.skey, nps);
  return nseg;
}

// one 8-byte piece of PW sources of one slot (layout at piece_srcs)
__device__ __forceinline__ uint2 make_piece(int order, uint32_t slot, const uint32_t* src)
{
  if (order == 1) {
    const uint64_t pc = (uint64_t)src[0] | (uint64_t)src[1] << kP1SrcBits | (uint64_t)src[2] << (2 * kP1SrcBits) |
                        (uint64_t)src[3] << (3 * kP1SrcBits) | (uint64_t)slot << kP1SlotShift;
    return make_uint2((uint32_t)pc, (uint32_t)(pc >> 32));
  }
  return make_uint2(src[0] | slot << kSrcBits, src[1] | slot << kSrcBits);
}

// Pass 1 (WRITE false): per chunk its padded vertex count, words and
// contributions.  Pass 2 (WRITE true): the chunk record and its words.
template <bool WRITE>
__global__ void __launch_bounds__(kSchedThreads) k_chunk(ChunkArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem& S = *reinterpret_cast<ChunkSmem*>(smem_raw);
  const int64_t ck = blockIdx.x;
  const int32_t b = A.cblk[ck], c = A.cpos[ck];
  const int CI = A.CI, nb = A.nb, nb2 = nb * nb;
  const int n_items = min(CI, A.item_count[b] - c * CI);
  const int32_t* it_ids = A.items + A.item_begin[b] + (int64_t)c * CI;
  const int nn = chunk_vertices(A, S, it_ids, n_items);
  const int nseg = chunk_segments(A, S, it_ids, n_items, b);
  const int nc = S.n_contrib;
  const int PW = A.order == 1 ? 4 : 2;
  // snake dealing: rank q to thread q % T (even rounds) or T - 1 - q % T (odd)
  const int T = kSchedThreads, t = threadIdx.x, lane = t & 31, w = t >> 5;
  auto seg_len = [&](int s) { return (s + 1 < nseg ? S.scan[s + 1] : nc) - S.scan[s]; };
  int pieces = 0;
  for (int r = 0;; ++r) {
    const int q = r * T + ((r & 1) ? T - 1 - t : t);
    if (q >= nseg) break;
    pieces += (seg_len((int)(S.skey[q] & 0x1fff)) + PW - 1) / PW;
  }
  const int K = __reduce_max_sync(0xffffffffu, pieces);
  if (lane == 0) S.warp_k[w] = K;
  __syncthreads();
  if (t == 0) {
    int off = 0;
    for (int x = 0; x < kWarps; ++x) {
      S.warp_off[x] = off;
      off += 64 * S.warp_k[x];
    }
    S.warp_off[kWarps] = off;
  }
  __syncthreads();
  if constexpr (!WRITE) {
    if (t == 0) {
      A.n_nodes[ck] = nn;
      A.words[ck] = S.warp_off[kWarps];
      A.contrib[ck] = nc;
    }
  } else {
    // ---- the record (layout at ChunkDesc)
    unsigned char* rec = A.records + A.rec_off[ck];
    const int n4 = (n_items + 3) & ~3;
    if (t == 0) {
      ChunkDesc cd{};
      cd.word_begin = A.word_begin[ck];
      for (int x = 0; x <= kWarps; ++x) cd.warp_off[x] = S.warp_off[x];
      cd.n_nodes = nn;
      if (c + kRecStages < A.nchunks[b]) {
        cd.next_off16 = (int32_t)(A.rec_off[ck + kRecStages] / 16);
        cd.next_bytes = (int32_t)(A.rec_off[ck + kRecStages + 1] - A.rec_off[ck + kRecStages]);
      }
      *reinterpret_cast<ChunkDesc*>(rec) = cd;
    }
    int32_t* ids = reinterpret_cast<int32_t*>(rec + sizeof(ChunkDesc));
    uint16_t* lc = reinterpret_cast<uint16_t*>(rec + sizeof(ChunkDesc) + 4 * n4);
    for (int i = t; i < n4; i += T) ids[i] = it_ids[i] >= 0 ? A.rank[it_ids[i]] : -1;  // -1 past the items
    for (int p = t; p < 4 * n4; p += T) lc[p] = p < 4 * n_items ? S.local_of[p] : (uint16_t)0;
    float4* va = reinterpret_cast<float4*>(rec + sizeof(ChunkDesc) + 12 * n4);
    float4* vb = reinterpret_cast<float4*>(rec + sizeof(ChunkDesc) + 12 * n4 + 16 * nn);
    float* vc = reinterpret_cast<float*>(rec + sizeof(ChunkDesc) + 12 * n4 + 32 * nn);
    const double4_32a o = A.xyz[S.node_of[0]];
    for (int l = t; l < nn; l += T) {
      // r = x - origin (FP64), split exactly r = hi + mid + lo
      const double4_32a x = A.xyz[S.node_of[l]];
      const double rr[3] = {__dsub_rn(x.x, o.x), __dsub_rn(x.y, o.y), __dsub_rn(x.z, o.z)};
      float h[3], md[3], lo[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        h[k] = __double2float_rn(rr[k]);
        const double r1 = __dsub_rn(rr[k], (double)h[k]);
        md[k] = __double2float_rn(r1);
        lo[k] = __double2float_rn(__dsub_rn(r1, (double)md[k]));
      }
      va[l] = make_float4(h[0], h[1], h[2], md[0]);
      vb[l] = make_float4(md[1], md[2], lo[0], lo[1]);
      vc[l] = lo[2];
    }
    // ---- the words: this thread's segments in rank order, PW sources a piece
    const uint32_t zero_src = (uint32_t)(A.nu * CI);
    uint2* out = reinterpret_cast<uint2*>(A.entries + A.word_begin[ck] + S.warp_off[w]) + lane;
    int kk = 0;
    for (int r = 0;; ++r) {
      const int q = r * T + ((r & 1) ? T - 1 - t : t);
      if (q >= nseg) break;
      const int s = (int)(S.skey[q] & 0x1fff), st = S.scan[s], len = seg_len(s);
      const uint32_t slot = S.ckey[st] >> 12;
      for (int k0 = 0; k0 < len; k0 += PW) {
        uint32_t src[4];
        for (int u = 0; u < PW; ++u) {
          src[u] = zero_src;
          if (k0 + u < len) {
            const int cand = (int)(S.ckey[st + k0 + u] & 0xfff);
            const int it = cand / nb2, i = (cand / nb) % nb, j = cand % nb;
            src[u] = (uint32_t)(sym_idx(i, j, nb) * CI + it);
          }
        }
        out[(int64_t)kk * 32] = make_piece(A.order, slot, src);
        ++kk;
      }
    }
    const uint32_t zs[4] = {zero_src, zero_src, zero_src, zero_src};
    for (; kk < K; ++kk) out[(int64_t)kk * 32] = make_piece(A.order, (uint32_t)kAccMax, zs);
  }
}

// per owned row in schedule order: (accumulator base, CSR start - base); two
// padding entries follow (the kernel's aligned copies of a row range)
__global__ void k_row_meta(int64_t nd, const int32_t* __restrict__ rows, const int32_t* __restrict__ row_acc,
                           const int32_t* __restrict__ rowptr, int2* __restrict__ meta)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < nd) meta[k] = make_int2(row_acc[k], rowptr[rows[k]] - row_acc[k]);
  else if (k < nd + 2) meta[k] = make_int2(0, 0);
}



__global__ void k_dofs_morton(int64_t E, int nb, const int32_t* __restrict__ elem_order, const int32_t* __restrict__ dofs,
                              int32_t* __restrict__ out)
{
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < E * nb) out[q] = dofs[(int64_t)elem_order[q / nb] * nb + q % nb];
}

// slot of each row's diagonal; col - row as int16 where every entry fits (flag
// cleared otherwise)
__global__ void k_diag_coloff(int64_t nd, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                              int32_t* __restrict__ diag, int16_t* __restrict__ coloff, int* __restrict__ fits)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nd) return;
  int lo = rowptr[r], hi = rowptr[r + 1];
  const int s0 = lo;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (colind[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  diag[r] = lo;
  for (int k = s0; k < rowptr[r + 1]; ++k) {
    const int64_t d = (int64_t)colind[k] - r;
    if (d < INT16_MIN || d > INT16_MAX) atomicAnd(fits, 0);
    else coloff[k] = (int16_t)d;
  }
}


}  // namespace

}  // namespace mg

namespace mg {

namespace {

// Device buffers of one schedule build, freed on every exit path unless handed
// to the plan.
struct SchedBuffers {
  std::vector<void*> ptrs;
  template <typename T>
  mg_status alloc(T** p, int64_t n)
  {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) return cuda_error(e, "device schedule buffer");
    ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return MG_OK;
  }
  void keep(void* q) { ptrs.erase(std::remove(ptrs.begin(), ptrs.end(), q), ptrs.end()); }
  ~SchedBuffers()
  {
    for (void* q : ptrs) cudaFree(q);
  }
};

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, (n + 255) / 256); }

template <typename T>
mg_status download(std::vector<T>& h, const T* d, int64_t n, cudaStream_t st)
{
  h.resize(n);
  if (n > 0) MG_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  return MG_OK;
}
template <typename T>
mg_status upload_to(SchedBuffers& B, T** d, const std::vector<T>& h, cudaStream_t st)
{
  MG_TRY(B.alloc(d, (int64_t)h.size()));
  if (!h.empty()) MG_CUDA(cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
  return MG_OK;
}

}  // namespace

// SMs of the current device (one persistent assembly CTA each); GB300's 152
// when the attribute is unavailable -- the same count the host build uses.
int64_t schedule_sm_count()
{
  int n = 0, dev = 0, sms = 0;
  if (cudaGetDeviceCount(&n) == cudaSuccess && n > 0 && cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
    return sms;
  cudaGetLastError();
  return 152;
}

mg_status build_schedule_device(mg_plan* p, cudaStream_t st)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb, order = m->order, CI = chunk_items(order), nu = nunique(order);
  const int64_t E = m->n_elem, nd = p->ndof, N = m->n_nodes;
  if (!p->d_rowptr || !p->d_colind) return set_error(MG_ERR_INVALID_ARG, "device schedule: pattern not on the device");
  if ((int64_t)CI * nb * nb > kMaxContrib || 4 * CI > kMaxRefs) return set_error(MG_ERR_SIZE, "device schedule: chunk size");
  if (nd >= INT32_MAX / 2 || E * nb >= INT32_MAX) return set_error(MG_ERR_SIZE, "device schedule: sizes above 2^30");
  MG_TRY(mesh_device(m));
  SchedBuffers B;
  // ---- 1. dofs along the Morton curve of their positions
  Box bx;
  for (int k = 0; k < 3; ++k) bx.lo[k] = INFINITY, bx.hi[k] = -INFINITY;
  for (int64_t i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) {
      bx.lo[k] = std::min(bx.lo[k], m->xyz[3 * i + k]);
      bx.hi[k] = std::max(bx.hi[k], m->xyz[3 * i + k]);
    }
  int32_t* d_edges = nullptr;
  if (nd > N) MG_TRY(upload_to(B, &d_edges, m->edge_nodes, st));
  const int64_t nmax = std::max(nd, E);
  uint64_t *ka, *kb;
  int32_t *ia, *ib;
  MG_TRY(B.alloc(&ka, nmax));
  MG_TRY(B.alloc(&kb, nmax));
  MG_TRY(B.alloc(&ia, nmax));
  MG_TRY(B.alloc(&ib, nmax));
  // CUB temporary storage: the largest of the sorts and scans below
  size_t tb = 0, q = 0;
  int64_t* i64a = nullptr;
  int32_t* i32a = nullptr;
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, q, ka, kb, ia, ib, (int)nmax, 0, 64, st));
  tb = std::max(tb, q);
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, q, i64a, i64a, (int)(nmax + 1), st));
  tb = std::max(tb, q);
  MG_CUDA(cub::DeviceScan::InclusiveSum(nullptr, q, i32a, i32a, (int)(nmax + 1), st));
  tb = std::max(tb, q);
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, q, i32a, i32a, (int)(nmax + 1), st));
  tb = std::max(tb, q);
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, q, i32a, i64a, (int)(nmax + 1), st));
  tb = std::max(tb, q);
  const int64_t items_cap = E * std::min(nb, 10);
  MG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, q, ka, kb, (int)std::max<int64_t>(items_cap, nmax), 0, 64, st));
  tb = std::max(tb, q);
  void* tmp = nullptr;
  MG_TRY(B.alloc(reinterpret_cast<unsigned char**>(&tmp), (int64_t)tb));
  const int g_nd = grid_of(nd), g_E = grid_of(E);
  k_dof_keys<<<g_nd, 256, 0, st>>>(nd, N, m->d_xyz, d_edges, bx, ka, ia);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, ka, kb, ia, ib, (int)nd, 0, 64, st));
  int32_t* d_order = ib;  // dof at Morton position t
  // ---- 2. blocks by prefix sums of the row weights
  int64_t *w, *wex;
  MG_TRY(B.alloc(&w, nd + 1));
  MG_TRY(B.alloc(&wex, nd + 1));
  k_weights<<<g_nd, 256, 0, st>>>(nd, d_order, p->d_rowptr, w);
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, w, wex, (int)nd, st));
  int64_t wtot = 0, wmax = 0;  // from the host copy of the pattern
  for (int64_t r = 0; r < nd; ++r) {
    const int64_t wr = std::max(p->rowptr[r + 1] - p->rowptr[r], 4);
    wtot += wr;
    wmax = std::max(wmax, wr);
  }
  const int64_t nbk_raw = schedule_block_count(wtot, wmax, schedule_sm_count());
  int32_t *flag, *incl, *bstart, *block_of_rank, *block_of;
  uint64_t* rowkeys;
  MG_TRY(B.alloc(&flag, nd));
  MG_TRY(B.alloc(&incl, nd));
  MG_TRY(B.alloc(&bstart, nbk_raw + 1));
  MG_TRY(B.alloc(&block_of_rank, nd));
  MG_TRY(B.alloc(&block_of, nd));
  MG_TRY(B.alloc(&rowkeys, nd));
  k_block_flags<<<g_nd, 256, 0, st>>>(nd, wex, wtot, nbk_raw, flag);
  MG_CUDA(cub::DeviceScan::InclusiveSum(tmp, tb, flag, incl, (int)nd, st));
  int32_t nbk = 0;
  MG_CUDA(cudaMemcpyAsync(&nbk, incl + nd - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  k_blocks_of<<<g_nd, 256, 0, st>>>(nd, d_order, incl, bstart, block_of_rank, block_of, rowkeys);
  MG_CUDA(cudaStreamSynchronize(st));
  // ---- 3. owned rows per block ascending; accumulator bases
  int bbits = 1;
  while ((1ll << bbits) <= nbk) ++bbits;
  MG_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, rowkeys, ka, (int)nd, 0, 32 + bbits, st));
  int32_t *rows, *lens, *accex, *row_acc, *row_acc_of;
  MG_TRY(B.alloc(&rows, nd));
  MG_TRY(B.alloc(&lens, nd + 1));
  MG_TRY(B.alloc(&accex, nd + 1));
  MG_TRY(B.alloc(&row_acc, nd));
  MG_TRY(B.alloc(&row_acc_of, nd));
  k_row_lens<<<g_nd, 256, 0, st>>>(nd, ka, p->d_rowptr, rows, lens);
  MG_CUDA(cudaMemsetAsync(lens + nd, 0, sizeof(int32_t), st));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, lens, accex, (int)(nd + 1), st));
  k_row_acc<<<g_nd, 256, 0, st>>>(nd, rows, accex, bstart, block_of_rank, row_acc, row_acc_of);
  // ---- 4. elements along the Morton curve of their centroids; items
  k_elem_keys<<<g_E, 256, 0, st>>>(E, m->d_conn, m->d_xyz, bx, ka, ia);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, ka, kb, ia, ib, (int)E, 0, 64, st));
  int32_t* d_elem_order;
  int32_t* rank;
  MG_TRY(B.alloc(&d_elem_order, E));
  MG_TRY(B.alloc(&rank, E));
  MG_CUDA(cudaMemcpyAsync(d_elem_order, ib, sizeof(int32_t) * E, cudaMemcpyDeviceToDevice, st));
  k_rank_of<<<g_E, 256, 0, st>>>(E, d_elem_order, rank);
  int32_t *icnt, *bcount;
  int64_t* ioff;
  MG_TRY(B.alloc(&icnt, E + 1));
  MG_TRY(B.alloc(&ioff, E + 1));
  MG_TRY(B.alloc(&bcount, nbk));
  k_item_counts<<<g_E, 256, 0, st>>>(E, nb, m->d_dofs, block_of, icnt);
  MG_CUDA(cudaMemsetAsync(icnt + E, 0, sizeof(int32_t), st));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, icnt, ioff, (int)(E + 1), st));
  int64_t n_items = 0;
  MG_CUDA(cudaMemcpyAsync(&n_items, ioff + E, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  if (n_items >= INT32_MAX / 2) return set_error(MG_ERR_SIZE, "assembly items above 2^30");
  uint64_t *ikeys, *ikeys2;
  MG_TRY(B.alloc(&ikeys, n_items));
  MG_TRY(B.alloc(&ikeys2, n_items));
  MG_CUDA(cudaMemsetAsync(bcount, 0, sizeof(int32_t) * nbk, st));
  k_item_keys<<<g_E, 256, 0, st>>>(E, nb, m->d_dofs, block_of, ioff, rank, ikeys, bcount);
  MG_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, ikeys, ikeys2, (int)n_items, 0, 32 + bbits, st));
  // per block (small arrays, on the host): padded item lists, chunks
  std::vector<int32_t> h_bcount, h_bstart;
  MG_TRY(download(h_bcount, bcount, nbk, st));
  MG_TRY(download(h_bstart, bstart, nbk, st));
  MG_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> cnt_ex(nbk + 1, 0), item_begin64(nbk + 1, 0);
  std::vector<int32_t> h_item_begin(nbk), h_nchunks(nbk), h_chunk_begin(nbk);
  int64_t nchunk_tot = 0;
  for (int32_t b = 0; b < nbk; ++b) {
    cnt_ex[b + 1] = cnt_ex[b] + h_bcount[b];
    item_begin64[b + 1] = item_begin64[b] + ((h_bcount[b] + 3) & ~3);
    h_item_begin[b] = (int32_t)item_begin64[b];
    h_nchunks[b] = (h_bcount[b] + CI - 1) / CI;
    h_chunk_begin[b] = (int32_t)nchunk_tot;
    nchunk_tot += h_nchunks[b];
  }
  const int64_t n_slots = item_begin64[nbk];
  if (n_slots >= INT32_MAX || nchunk_tot >= INT32_MAX / 2) return set_error(MG_ERR_SIZE, "assembly items above 2^31-1");
  int64_t *d_cnt_ex, *d_item_begin64;
  int32_t *d_items, *d_item_begin, *d_nchunks, *d_chunk_begin;
  MG_TRY(upload_to(B, &d_cnt_ex, cnt_ex, st));
  MG_TRY(upload_to(B, &d_item_begin64, item_begin64, st));
  MG_TRY(upload_to(B, &d_item_begin, h_item_begin, st));
  MG_TRY(upload_to(B, &d_nchunks, h_nchunks, st));
  MG_TRY(upload_to(B, &d_chunk_begin, h_chunk_begin, st));
  MG_TRY(B.alloc(&d_items, n_slots));
  MG_CUDA(cudaMemsetAsync(d_items, 0xff, sizeof(int32_t) * std::max<int64_t>(n_slots, 1), st));  // -1 padding
  k_items_place<<<grid_of(n_items), 256, 0, st>>>(n_items, ikeys2, d_elem_order, d_cnt_ex, d_item_begin64, d_items);
  int32_t *cblk, *cpos;
  MG_TRY(B.alloc(&cblk, nchunk_tot));
  MG_TRY(B.alloc(&cpos, nchunk_tot));
  k_chunk_owner<<<grid_of(nbk), 256, 0, st>>>(nbk, d_chunk_begin, d_nchunks, cblk, cpos);
  // ---- 5. per chunk: pass 1 (counts), host scans, pass 2 (records and words)
  ChunkArgs A{};
  A.order = order, A.nb = nb, A.CI = CI, A.nu = nu;
  A.items = d_items, A.rank = rank, A.item_begin = d_item_begin, A.item_count = bcount, A.nchunks = d_nchunks;
  A.cblk = cblk, A.cpos = cpos;
  A.conn = m->d_conn, A.dofs = m->d_dofs, A.block_of = block_of, A.row_acc_of = row_acc_of;
  A.rowptr = p->d_rowptr, A.colind = p->d_colind, A.xyz = m->d_xyz;
  int64_t *c_words, *c_contrib;
  int32_t* c_nodes;
  MG_TRY(B.alloc(&c_words, nchunk_tot));
  MG_TRY(B.alloc(&c_contrib, nchunk_tot));
  MG_TRY(B.alloc(&c_nodes, nchunk_tot));
  A.n_nodes = c_nodes, A.words = c_words, A.contrib = c_contrib;
  const size_t csmem = sizeof(ChunkSmem);
  MG_CUDA(cudaFuncSetAttribute(k_chunk<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem));
  MG_CUDA(cudaFuncSetAttribute(k_chunk<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem));
  if (nchunk_tot > 0) k_chunk<false><<<(unsigned)nchunk_tot, kSchedThreads, csmem, st>>>(A);
  MG_CUDA(cudaGetLastError());
  std::vector<int64_t> h_words, h_contrib;
  std::vector<int32_t> h_nodes, h_cblk;
  MG_TRY(download(h_words, c_words, nchunk_tot, st));
  MG_TRY(download(h_contrib, c_contrib, nchunk_tot, st));
  MG_TRY(download(h_nodes, c_nodes, nchunk_tot, st));
  MG_TRY(download(h_cblk, cblk, nchunk_tot, st));
  MG_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> word_begin(nchunk_tot + 1, 0), rec_off(nchunk_tot + 1, 0);
  int64_t n_contrib = 0, max_words = 0, max_rec = 0;
  int32_t max_nodes = 0;
  for (int64_t ck = 0; ck < nchunk_tot; ++ck) {
    const int32_t b = h_cblk[ck];
    const int64_t c = ck - h_chunk_begin[b];
    const int64_t n4 = (std::min<int64_t>(CI, h_bcount[b] - c * CI) + 3) & ~3;
    const int64_t bytes = (int64_t)sizeof(ChunkDesc) + 12 * n4 + 36 * (int64_t)h_nodes[ck];
    word_begin[ck + 1] = word_begin[ck] + h_words[ck];
    rec_off[ck + 1] = rec_off[ck] + bytes;
    n_contrib += h_contrib[ck];
    max_words = std::max(max_words, h_words[ck]);
    max_rec = std::max(max_rec, bytes);
    max_nodes = std::max(max_nodes, h_nodes[ck]);
  }
  if (max_nodes > 65535) return set_error(MG_ERR_SIZE, "a chunk touches more than 65535 vertices");
  if (rec_off[nchunk_tot] / 16 >= INT32_MAX || max_rec >= INT32_MAX) return set_error(MG_ERR_SIZE, "chunk records above 32 GiB");
  if (word_begin[nchunk_tot] / 32 >= INT32_MAX) return set_error(MG_ERR_SIZE, "contribution words above 2^36");
  int64_t *d_word_begin, *d_rec_off;
  unsigned char* d_records;
  uint32_t* d_entries;
  MG_TRY(upload_to(B, &d_word_begin, word_begin, st));
  MG_TRY(upload_to(B, &d_rec_off, rec_off, st));
  MG_TRY(B.alloc(&d_records, std::max<int64_t>(rec_off[nchunk_tot], 16)));
  MG_TRY(B.alloc(&d_entries, word_begin[nchunk_tot]));
  A.word_begin = d_word_begin, A.rec_off = d_rec_off, A.records = d_records, A.entries = d_entries;
  if (nchunk_tot > 0) k_chunk<true><<<(unsigned)nchunk_tot, kSchedThreads, csmem, st>>>(A);
  MG_CUDA(cudaGetLastError());
  std::vector<int2> h_rec(nchunk_tot);
  for (int64_t ck = 0; ck < nchunk_tot; ++ck)
    h_rec[ck] = make_int2((int32_t)(rec_off[ck] / 16), (int32_t)(rec_off[ck + 1] - rec_off[ck]));
  int2* d_rec;
  MG_TRY(upload_to(B, &d_rec, h_rec, st));
  // ---- block descriptors, in Morton order of their rows (as the host builder)
  std::vector<BlockDesc> blocks(nbk);
  {
    std::vector<int32_t> h_accex;
    MG_TRY(download(h_accex, accex, nd + 1, st));
    MG_CUDA(cudaStreamSynchronize(st));
    for (int32_t b = 0; b < nbk; ++b) {
      BlockDesc& d = blocks[b];
      d.item_begin = h_item_begin[b];
      d.item_count = h_bcount[b];
      d.chunk_begin = h_chunk_begin[b];
      d.nchunks = h_nchunks[b];
      d.row_begin = h_bstart[b];
      const int32_t r1 = b + 1 < nbk ? h_bstart[b + 1] : (int32_t)nd;
      d.row_count = r1 - h_bstart[b];
      d.acc_used = h_accex[r1] - h_accex[h_bstart[b]];
      d.word_begin32 = (int32_t)(word_begin[h_chunk_begin[b]] / 32);
    }
  }
  BlockDesc* d_blocks;
  MG_TRY(upload_to(B, &d_blocks, blocks, st));
  // ---- row metadata, element order, dofs in that order, diagonal, 16-bit columns
  int2* d_meta;
  MG_TRY(B.alloc(&d_meta, nd + 2));
  k_row_meta<<<grid_of(nd + 2), 256, 0, st>>>(nd, rows, row_acc, p->d_rowptr, d_meta);
  int32_t* d_dm;
  MG_TRY(B.alloc(&d_dm, E * nb));
  k_dofs_morton<<<grid_of(E * nb), 256, 0, st>>>(E, nb, d_elem_order, m->d_dofs, d_dm);
  int32_t* d_diag;
  int16_t* d_coloff;
  int* d_fits;
  MG_TRY(B.alloc(&d_diag, nd));
  MG_TRY(B.alloc(&d_coloff, p->nnz));
  MG_TRY(B.alloc(&d_fits, 1));
  const int one = 1;
  MG_CUDA(cudaMemcpyAsync(d_fits, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  k_diag_coloff<<<g_nd, 256, 0, st>>>(nd, p->d_rowptr, p->d_colind, d_diag, d_coloff, d_fits);
  MG_CUDA(cudaGetLastError());
  int fits = 0;
  MG_CUDA(cudaMemcpyAsync(&fits, d_fits, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_TRY(download(p->h_elem_order, d_elem_order, E, st));
  MG_CUDA(cudaStreamSynchronize(st));
  // ---- into the plan (the host build's plan_device state)
  uint32_t* d_counters;
  MG_TRY(upload_to(B, &d_counters, std::vector<uint32_t>(8, 0u), st));
  MG_CUDA(cudaMallocHost(&p->h_pinned, 64 * sizeof(double)));
  MG_CUDA(cudaStreamSynchronize(st));
  p->d_diag = d_diag;
  p->d_coloff = (fits && p->nnz > 0) ? d_coloff : nullptr;
  p->d_blocks = d_blocks;
  p->d_entries = d_entries;
  p->d_elem_order = d_elem_order;
  p->d_dofs_morton = d_dm;
  p->d_row_meta = d_meta;
  p->d_chunk_data = d_records;
  p->d_chunk_rec = d_rec;
  p->d_chunk_wb = d_word_begin;
  p->d_counters = d_counters;
  p->d_sched_rows = rows;
  for (void* q : {(void*)rows, (void*)d_diag, (void*)d_blocks, (void*)d_entries, (void*)d_elem_order, (void*)d_dm, (void*)d_meta,
                  (void*)d_records, (void*)d_rec, (void*)d_word_begin, (void*)d_counters})
    B.keep(q);
  if (p->d_coloff) B.keep(d_coloff);
  p->nblocks = nbk;
  p->n_items = n_items;
  p->n_item_slots = n_slots;
  p->n_chunks = nchunk_tot;
  p->n_entries = word_begin[nchunk_tot];
  p->n_contrib = n_contrib;
  p->max_chunk_entries = max_words;
  p->max_chunk_nodes = max_nodes;
  p->max_rec_bytes = (int32_t)max_rec;
  p->on_device = true;
  return MG_OK;
}

}  // namespace mg
