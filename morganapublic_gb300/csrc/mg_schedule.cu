// Plan set-up on the GPU: the element order of the assembly, the slot map of its
// gather, and the CSR helpers (diagonal entries, 16-bit column offsets).
//   1. elements along a Morton curve of their centroids: 64-bit keys,
//      radix-sorted with the element id (ties by id) -- the host build
//      (mg_plan.cpp) computes the same keys and order;
//   2. the slot map (build_slot_map): for every diagonal or upper CSR entry the
//      element-matrix entries summed into it, in ascending Morton position;
//      laid out for the two-pass gather (P2) or turned into the block map of
//      the one-pass assembly (P1, build_block_map).
// Setup-only library calls: CUB radix sorts and scans.
#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "mg_internal.h"

namespace mg {

namespace {

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

// Device buffers of one plan build, freed on every exit path unless handed
// to the plan.
struct SchedBuffers {
  std::vector<void*> ptrs;
  template <typename T>
  mg_status alloc(T** p, int64_t n)
  {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) return cuda_error(e, "device plan buffer");
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

// Every operator of the path is symmetric, and the contributions to CSR entries
// (r, c) and (c, r) are the same element-matrix entries (the element's unique
// pair u), summed in the same order: the values are bitwise equal.  The gather
// therefore sums each diagonal and upper entry (c >= r) once and writes it to
// both places.  For upper entry t (CSR order):
//   uslot[t]   the CSR entry (r, c);  umirror[t] the entry (c, r) (= uslot[t] on
//              the diagonal)
//   src[useg[t] .. useg[t+1])  the element-matrix entries summed into it, one per
//              element holding both dofs, ascending Morton position p; each the
//              index of (p, u) in the element-matrix array: p * nu + u
//              (element-major, P1) or u * E + p (entry-major, P2).
// Built from the plan's Morton dofs and device pattern:
//   1. incidence: (dof, q = p nb + l) pairs radix-sorted by dof (stable, so each
//      dof's list ascends in q, hence in p);
//   2. one thread per row: its upper entries and their contributions counted;
//      exclusive scans give each row's first upper entry and first source;
//   3. one thread per row: per-entry counts (a binary search of each coupled
//      column in the row), their prefix, then the sources in incidence order.

__global__ void k_iota32(int64_t n, uint32_t* v)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

// ptr[d] = first t with (key[t] >> shift) >= d, d = 0 .. nkeys (keys sorted ascending)
__global__ void k_run_starts(int64_t n, const uint32_t* key, int64_t nkeys, int32_t* ptr, int shift = 0)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t > n) return;
  const int64_t lo = t == 0 ? 0 : (int64_t)(key[t - 1] >> shift) + 1;
  const int64_t hi = t == n ? nkeys : (int64_t)(key[t] >> shift);
  for (int64_t d = lo; d <= hi; ++d) ptr[d] = (int32_t)t;
}

// position of `col` in the sorted columns c[0 .. len)
__device__ __forceinline__ int find_col(const int32_t* c, int len, int32_t col)
{
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (c[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// per row: upper entries (c >= r) and the contributions they receive
__global__ void __launch_bounds__(256) k_upper_counts(int64_t nd, int nb, const int32_t* __restrict__ inc_ptr,
                                                      const uint32_t* __restrict__ inc_q,
                                                      const int32_t* __restrict__ dofs_m,
                                                      const int32_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ colind, int32_t* n_upper,
                                                      int32_t* n_contrib)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nd) return;
  const int32_t r0 = rowptr[r], len = rowptr[r + 1] - r0;
  n_upper[r] = len - find_col(colind + r0, len, (int32_t)r);
  int32_t c = 0;
  for (int32_t t = inc_ptr[r]; t < inc_ptr[r + 1]; ++t) {
    const int64_t p = inc_q[t] / nb;
    for (int j = 0; j < nb; ++j) c += dofs_m[p * nb + j] >= r ? 1 : 0;
  }
  n_contrib[r] = c;
}

__global__ void __launch_bounds__(256) k_slot_map(int64_t nd, int nb, int64_t E, int aos,
                                                  const int32_t* __restrict__ inc_ptr,
                                                  const uint32_t* __restrict__ inc_q, const int32_t* __restrict__ dofs_m,
                                                  const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                                  const int32_t* __restrict__ up_first,
                                                  const int32_t* __restrict__ src_first, int32_t* cur, int32_t* useg,
                                                  int32_t* uslot, int32_t* umirror, int32_t* urow, uint32_t* src,
                                                  int* bad)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nd) return;
  const int32_t r0 = rowptr[r], len = rowptr[r + 1] - r0;
  const int32_t* cols = colind + r0;
  const int kd = find_col(cols, len, (int32_t)r);  // first upper entry of the row
  const int32_t i0 = inc_ptr[r], i1 = inc_ptr[r + 1], u0 = up_first[r];
  const int nu = nb * (nb + 1) / 2;
  for (int k = kd; k < len; ++k) cur[r0 + k] = 0;
  for (int32_t t = i0; t < i1; ++t) {
    const int64_t p = inc_q[t] / nb;
    for (int j = 0; j < nb; ++j) {
      const int32_t col = dofs_m[p * nb + j];
      if (col < r) continue;
      const int k = find_col(cols, len, col);
      if (k >= len || cols[k] != col) {
        *bad = 1;
        return;
      }
      cur[r0 + k]++;
    }
  }
  int32_t pos = src_first[r];
  for (int k = kd; k < len; ++k) {
    const int32_t c = cur[r0 + k];
    const int32_t t = u0 + (k - kd);
    useg[t] = pos;
    uslot[t] = r0 + k;
    urow[t] = (int32_t)r;
    const int32_t col = cols[k];
    const int32_t m0 = rowptr[col], ml = rowptr[col + 1] - m0;
    const int km = find_col(colind + m0, ml, (int32_t)r);
    if (km >= ml || colind[m0 + km] != (int32_t)r) {
      *bad = 1;
      return;
    }
    umirror[t] = m0 + km;
    cur[r0 + k] = pos;
    pos += c;
  }
  for (int32_t t = i0; t < i1; ++t) {
    const uint32_t q = inc_q[t];
    const int64_t p = q / nb;
    const int l = (int)(q - p * nb);
    for (int j = 0; j < nb; ++j) {
      const int32_t col = dofs_m[p * nb + j];
      if (col < r) continue;
      const int k = find_col(cols, len, col);
      const int u = sym_index(l, j, nb);
      src[cur[r0 + k]++] = aos ? (uint32_t)(p * nu + u) : (uint32_t)(u * E + p);
    }
  }
}


// ---- the gather's layout: upper entries regrouped (diagonal entries first, each
// class in CSR order) into groups of 32, one per warp; a group's sources stored
// [j][lane], padded to its longest list with kPadSource
// key of upper entry t in the gather's order: (row / kGatherRowBlock, off-diagonal)
__global__ void k_group_keys(int64_t U, const int32_t* __restrict__ urow, const int32_t* __restrict__ uslot,
                             const int32_t* __restrict__ umirror, uint32_t* __restrict__ key, uint32_t* __restrict__ id,
                             int32_t* __restrict__ ndiag)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= U) return;
  const bool dg = uslot[t] == umirror[t];
  key[t] = ((uint32_t)(urow[t] / kGatherRowBlock) << 1) | (dg ? 0u : 1u);
  id[t] = (uint32_t)t;
  if (dg) atomicAdd(ndiag, 1);
}

__global__ void k_group_len(int64_t G, int64_t U, const uint32_t* __restrict__ perm, const int32_t* __restrict__ useg,
                            int32_t* __restrict__ glen)
{
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g > G) return;
  int32_t L = 0;
  if (g < G)
    for (int64_t t = 32 * g; t < min(32 * g + 32, U); ++t) {
      const uint32_t q = perm[t];
      L = max(L, useg[q + 1] - useg[q]);
    }
  glen[g] = 32 * L;
}

__global__ void k_narrow(int64_t n, const int64_t* __restrict__ a, int32_t* __restrict__ b)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (int32_t)a[i];
}

__global__ void k_group_fill(int64_t G, int64_t U, const uint32_t* __restrict__ perm, const int32_t* __restrict__ useg,
                             const uint32_t* __restrict__ src_in, const int32_t* __restrict__ uslot_in,
                             const int32_t* __restrict__ umirror_in, const int32_t* __restrict__ goff,
                             uint32_t* __restrict__ src, int32_t* __restrict__ uslot, int32_t* __restrict__ umirror)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= 32 * G) return;
  const int64_t g = t >> 5;
  const int lane = (int)(t & 31);
  const int32_t o = goff[g], L = (goff[g + 1] - o) >> 5;
  int32_t s0 = 0, len = 0;
  if (t < U) {
    const uint32_t q = perm[t];
    s0 = useg[q];
    len = useg[q + 1] - s0;
    uslot[t] = uslot_in[q];
    umirror[t] = umirror_in[q];
  }
  for (int32_t j = 0; j < L; ++j) src[o + 32 * j + lane] = j < len ? src_in[s0 + j] : kPadSource;
}


// ---- the block map of the one-pass P1 assembly (see mg_plan::d_bgrp).  A run
// is a maximal stretch of an upper entry's sources (ascending p) in one element
// block; an entry with one run is complete, else shared, its runs numbered j in
// ascending block.  An entry without sources (not produced by a mesh's pattern)
// counts as one empty run of block 0, so that its value is written (zero).
__device__ __forceinline__ int32_t block_of(uint32_t s, int nu, int be) { return (int32_t)(s / (uint32_t)nu / be); }

__global__ void k_run_count(int64_t U, int nu, int be, const int32_t* __restrict__ useg,
                            const uint32_t* __restrict__ src, int32_t* __restrict__ nrun, int32_t* __restrict__ shared)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t > U) return;
  if (t == U) {  // the exclusive scans' last entry
    nrun[U] = 0;
    shared[U] = 0;
    return;
  }
  int32_t n = 0, prev = -1;
  for (int32_t k = useg[t]; k < useg[t + 1]; ++k) {
    const int32_t b = block_of(src[k], nu, be);
    if (b != prev) ++n, prev = b;
  }
  n = max(n, 1);
  nrun[t] = n;
  shared[t] = n > 1 ? 1 : 0;
}

// per run: sort key 64 b + 63 - min(length, 63) (per block the longest runs
// first, so that a group's lanes have similar lengths), its entry, rank, first
// source, length
__device__ __forceinline__ uint32_t run_key(int32_t b, int32_t len)
{
  return 64u * (uint32_t)b + 63u - (uint32_t)min(len, 63);
}

__global__ void k_run_emit(int64_t U, int nu, int be, const int32_t* __restrict__ useg,
                           const uint32_t* __restrict__ src,
                           const int32_t* __restrict__ rfirst, uint32_t* __restrict__ rkey, uint32_t* __restrict__ rid,
                           int32_t* __restrict__ rt, int32_t* __restrict__ rj, int32_t* __restrict__ rstart,
                           int32_t* __restrict__ rlen)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= U) return;
  const int32_t k0 = useg[t], k1 = useg[t + 1];
  int32_t ri = rfirst[t], j = 0;
  if (k0 == k1) {
    rkey[ri] = run_key(0, 0), rid[ri] = (uint32_t)ri, rt[ri] = (int32_t)t, rj[ri] = 0, rstart[ri] = k0, rlen[ri] = 0;
    return;
  }
  for (int32_t k = k0; k < k1;) {
    const int32_t b = block_of(src[k], nu, be);
    int32_t e = k + 1;
    while (e < k1 && block_of(src[e], nu, be) == b) ++e;
    rkey[ri] = run_key(b, e - k);
    rid[ri] = (uint32_t)ri;
    rt[ri] = (int32_t)t;
    rj[ri] = j++;
    rstart[ri] = k;
    rlen[ri] = e - k;
    ++ri;
    k = e;
  }
}

// groups of 32 runs per block: their count, then each group's first sorted run
// and lane count
__global__ void k_seg_groups(int64_t nseg, const int32_t* __restrict__ seg_ptr, int32_t* __restrict__ ng)
{
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < nseg) ng[s] = (seg_ptr[s + 1] - seg_ptr[s] + 31) / 32;
  else if (s == nseg) ng[s] = 0;
}

__global__ void k_seg_fill(int64_t nseg, const int32_t* __restrict__ seg_ptr, const int32_t* __restrict__ seg_g,
                           int32_t* __restrict__ grun0, int32_t* __restrict__ gcnt)
{
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int32_t r0 = seg_ptr[s], r1 = seg_ptr[s + 1];
  for (int32_t g = seg_g[s], r = r0; r < r1; ++g, r += 32) {
    grun0[g] = r;
    gcnt[g] = min(32, r1 - r);
  }
}

// 32 x the longest run of each group (the [j][lane] rows of its sources)
__global__ void k_bgroup_len(int64_t G, const int32_t* __restrict__ grun0, const int32_t* __restrict__ gcnt,
                             const uint32_t* __restrict__ perm, const int32_t* __restrict__ rlen,
                             int32_t* __restrict__ glen)
{
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g > G) return;
  int32_t L = 0;
  if (g < G)
    for (int32_t l = 0; l < gcnt[g]; ++l) L = max(L, rlen[perm[grun0[g] + l]]);
  glen[g] = 32 * L;
}

// the shared entries in CSR order, and 32 x the most runs of each group of 32
__global__ void k_shared_list(int64_t U, const int32_t* __restrict__ shared, const int32_t* __restrict__ sidx,
                              int32_t* __restrict__ sh_t)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < U && shared[t]) sh_t[sidx[t]] = (int32_t)t;
}

// shared entry i (CSR order) keyed by its run count, most first; and the
// inverse of the sorted order
__global__ void k_shared_keys(int64_t S, const int32_t* __restrict__ sh_t, const int32_t* __restrict__ nrun,
                              uint32_t* __restrict__ key)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < S) key[i] = 63u - (uint32_t)min(nrun[sh_t[i]], 63);
}

__global__ void k_shared_rank(int64_t S, const int32_t* __restrict__ sh_sorted, int32_t* __restrict__ srank)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < S) srank[sh_sorted[i]] = (int32_t)i;
}

__global__ void k_sgroup_len(int64_t G3, int64_t S, const int32_t* __restrict__ sh_t, const int32_t* __restrict__ nrun,
                             int32_t* __restrict__ slen)
{
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g > G3) return;
  int32_t L = 0;
  if (g < G3)
    for (int64_t i = 32 * g; i < min(32 * g + 32, S); ++i) L = max(L, nrun[sh_t[i]]);
  slen[g] = 32 * L;
}

__global__ void k_sgroup_out(int64_t G3, int64_t S, const int32_t* __restrict__ sh_t, const int32_t* __restrict__ uslot,
                             const int32_t* __restrict__ umirror, int2* __restrict__ sout)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 32 * G3) return;
  sout[i] = i < S ? make_int2(uslot[sh_t[i]], umirror[sh_t[i]]) : make_int2(kNoOutput, kNoOutput);
}

// one thread per (group, lane): the run's local sources [j][lane] and its output
__global__ void k_bfill(int64_t G, int nu, int be, const int32_t* __restrict__ grun0, const int32_t* __restrict__ gcnt,
                        const uint32_t* __restrict__ perm, const uint32_t* __restrict__ skey,
                        const int32_t* __restrict__ rt, const int32_t* __restrict__ rj,
                        const int32_t* __restrict__ rstart, const int32_t* __restrict__ rlen,
                        const uint32_t* __restrict__ src, const int32_t* __restrict__ uslot,
                        const int32_t* __restrict__ umirror, const int32_t* __restrict__ nrun,
                        const int32_t* __restrict__ srank, const int32_t* __restrict__ sgoff,
                        const int32_t* __restrict__ bgoff, uint16_t* __restrict__ bsrc, int2* __restrict__ bout)
{
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 32 * G) return;
  const int64_t g = i >> 5;
  const int lane = (int)(i & 31);
  const int32_t o = bgoff[g], L = (bgoff[g + 1] - o) >> 5;
  const uint16_t pad = (uint16_t)(be * nu);
  if (lane >= gcnt[g]) {
    bout[i] = make_int2(kNoOutput, 0);
    for (int32_t j = 0; j < L; ++j) bsrc[o + 32 * j + lane] = pad;
    return;
  }
  const int32_t sr = grun0[g] + lane;
  const uint32_t ri = perm[sr];
  const uint32_t base = (skey[sr] >> 6) * (uint32_t)be * (uint32_t)nu;
  const int32_t t = rt[ri], k0 = rstart[ri], len = rlen[ri];
  for (int32_t j = 0; j < L; ++j) bsrc[o + 32 * j + lane] = j < len ? (uint16_t)(src[k0 + j] - base) : pad;
  if (nrun[t] == 1) {
    bout[i] = make_int2(uslot[t], umirror[t]);
  } else {
    const int32_t s = srank[t];
    const int32_t q = sgoff[s >> 5] + 32 * rj[ri] + (s & 31);
    bout[i] = make_int2(-1 - q, 0);
  }
}

// block b's first group and first local source
__global__ void k_bgrp(int64_t nblk, const int32_t* __restrict__ seg_g, const int32_t* __restrict__ bgoff,
                       int32_t* __restrict__ bgrp, int32_t* __restrict__ bsrc0)
{
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b <= nblk) {
    bgrp[b] = seg_g[b];
    bsrc0[b] = bgoff[seg_g[b]];
  }
}

template <typename In, typename Out>
mg_status exclusive_scan(SchedBuffers& B, const In* in, Out* out, int64_t n, cudaStream_t st)
{
  size_t tb = 0;
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, (int)n, st));
  unsigned char* tmp;
  MG_TRY(B.alloc(&tmp, (int64_t)std::max(tb, (size_t)1)));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, (int)n, st));
  return MG_OK;
}

template <typename T>
mg_status read_back(T* h, const T* d, cudaStream_t st)
{
  MG_CUDA(cudaMemcpyAsync(h, d, sizeof(T), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  return MG_OK;
}

// 64-bit offsets narrowed to the plan's 32-bit layout, checked
mg_status narrow_offsets(SchedBuffers& B, const int32_t* len, int64_t n, int32_t** out, int64_t* total,
                         const char* what, cudaStream_t st)
{
  int64_t* off64;
  MG_TRY(B.alloc(&off64, n + 1));
  MG_TRY(exclusive_scan(B, len, off64, n + 1, st));
  MG_TRY(read_back(total, off64 + n, st));
  if (*total >= INT32_MAX) return set_error(MG_ERR_SIZE, std::string(what) + " above 2^31 entries");
  MG_TRY(B.alloc(out, n + 1));
  k_narrow<<<grid_of(n + 1), 256, 0, st>>>(n + 1, off64, *out);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace

// --------------------------------------------------------------- slot map --
// element-matrix layout of the gather assembly: element-major for P1
bool slot_map_aos(int order) { return order == 1; }

mg_status build_slot_map(mg_plan* p, cudaStream_t st)
{
  const mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = p->ndof, nnz = p->nnz, n = E * nb;
  if (n * nb >= INT32_MAX) return set_error(MG_ERR_SIZE, "slot map above 2^31 contributions");
  if ((int64_t)nunique(m->order) * E >= (int64_t)INT32_MAX)
    return set_error(MG_ERR_SIZE, "element matrices above 2^31 entries");
  SchedBuffers B;
  int32_t *inc_ptr, *cur, *nup, *ncon, *up_first, *src_first;
  uint32_t *keys, *vin, *vout;
  int* bad;
  MG_TRY(B.alloc(&inc_ptr, nd + 1));
  MG_TRY(B.alloc(&cur, nnz));
  MG_TRY(B.alloc(&nup, nd + 1));
  MG_TRY(B.alloc(&ncon, nd + 1));
  MG_TRY(B.alloc(&up_first, nd + 1));
  MG_TRY(B.alloc(&src_first, nd + 1));
  MG_TRY(B.alloc(&keys, n));
  MG_TRY(B.alloc(&vin, n));
  MG_TRY(B.alloc(&vout, n));
  MG_TRY(B.alloc(&bad, 1));
  MG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  int kbits = 1;
  while ((1ll << kbits) <= nd) ++kbits;
  size_t tb = 0, tb2 = 0;
  unsigned char* tmp = nullptr;
  const uint32_t* kin = reinterpret_cast<const uint32_t*>(p->d_dofs_morton);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, kin, keys, vin, vout, (int)n, 0, kbits, st));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb2, nup, up_first, (int)(nd + 1), st));
  MG_TRY(B.alloc(&tmp, (int64_t)std::max(tb, tb2)));
  tb = std::max(tb, tb2);
  k_iota32<<<grid_of(n), 256, 0, st>>>(n, vin);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, kin, keys, vin, vout, (int)n, 0, kbits, st));
  k_run_starts<<<grid_of(n + 1), 256, 0, st>>>(n, keys, nd, inc_ptr);
  k_upper_counts<<<grid_of(nd), 256, 0, st>>>(nd, nb, inc_ptr, vout, p->d_dofs_morton, p->d_rowptr, p->d_colind, nup,
                                               ncon);
  MG_CUDA(cudaMemsetAsync(nup + nd, 0, sizeof(int32_t), st));
  MG_CUDA(cudaMemsetAsync(ncon + nd, 0, sizeof(int32_t), st));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, nup, up_first, (int)(nd + 1), st));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, ncon, src_first, (int)(nd + 1), st));
  int32_t tot[2] = {0, 0};
  MG_CUDA(cudaMemcpyAsync(&tot[0], up_first + nd, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaMemcpyAsync(&tot[1], src_first + nd, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  const int64_t U = tot[0], C = tot[1];
  int32_t *useg, *uslot, *umirror, *urow;
  uint32_t* src;
  MG_TRY(B.alloc(&useg, U + 1));
  MG_TRY(B.alloc(&uslot, U));
  MG_TRY(B.alloc(&umirror, U));
  MG_TRY(B.alloc(&urow, U));
  MG_TRY(B.alloc(&src, C));
  k_slot_map<<<grid_of(nd), 256, 0, st>>>(nd, nb, E, slot_map_aos(m->order) ? 1 : 0, inc_ptr, vout,
                                           p->d_dofs_morton, p->d_rowptr, p->d_colind, up_first, src_first, cur, useg,
                                           uslot, umirror, urow, src, bad);
  const int32_t last = (int32_t)C;
  MG_CUDA(cudaMemcpyAsync(useg + U, &last, sizeof(int32_t), cudaMemcpyHostToDevice, st));
  MG_CUDA(cudaGetLastError());
  int hbad = 0;
  MG_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  if (hbad) return set_error(MG_ERR_INVALID_ARG, "slot map: an element coupling is missing from the plan's pattern");
  if (uses_block_map(m->order)) {
    // one-pass assembly: the per-entry lists become the block map
    MG_TRY(build_block_map(p, U, useg, uslot, umirror, src, st));
    p->n_upper = U;
    p->n_slot_contrib = C;
    return MG_OK;
  }
  // ---- regroup for the gather: entries stably sorted by (row block, off-diagonal)
  const int64_t G = (U + 31) / 32;
  int32_t *glen, *goff, *gslot, *gmirror, *d_ndiag;
  uint32_t *gkey, *gkey2, *gid, *perm, *gsrc;
  MG_TRY(B.alloc(&gkey, U));
  MG_TRY(B.alloc(&gkey2, U));
  MG_TRY(B.alloc(&gid, U));
  MG_TRY(B.alloc(&perm, U));
  MG_TRY(B.alloc(&glen, G + 1));
  MG_TRY(B.alloc(&goff, G + 1));
  MG_TRY(B.alloc(&gslot, U));
  MG_TRY(B.alloc(&gmirror, U));
  MG_TRY(B.alloc(&d_ndiag, 1));
  MG_CUDA(cudaMemsetAsync(d_ndiag, 0, sizeof(int32_t), st));
  int gbits = 1;
  while ((1ll << gbits) <= 2 * (nd / kGatherRowBlock + 1)) ++gbits;
  size_t tb3 = 0;
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb3, gkey, gkey2, gid, perm, (int)U, 0, gbits, st));
  unsigned char* tmp3;
  MG_TRY(B.alloc(&tmp3, (int64_t)std::max(tb3, (size_t)1)));
  if (U > 0) k_group_keys<<<grid_of(U), 256, 0, st>>>(U, urow, uslot, umirror, gkey, gid, d_ndiag);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp3, tb3, gkey, gkey2, gid, perm, (int)U, 0, gbits, st));
  int32_t ndiag = 0;
  MG_CUDA(cudaMemcpyAsync(&ndiag, d_ndiag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  k_group_len<<<grid_of(G + 1), 256, 0, st>>>(G, U, perm, useg, glen);
  // group offsets summed in 64 bits, checked against the 32-bit layout
  int64_t* goff64;
  MG_TRY(B.alloc(&goff64, G + 1));
  size_t tb4 = 0;
  MG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb4, glen, goff64, (int)(G + 1), st));
  unsigned char* tmp4;
  MG_TRY(B.alloc(&tmp4, (int64_t)std::max(tb4, (size_t)1)));
  MG_CUDA(cub::DeviceScan::ExclusiveSum(tmp4, tb4, glen, goff64, (int)(G + 1), st));
  int64_t S = 0;
  MG_CUDA(cudaMemcpyAsync(&S, goff64 + G, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  if (S >= INT32_MAX) return set_error(MG_ERR_SIZE, "slot map: padded sources above 2^31");
  k_narrow<<<grid_of(G + 1), 256, 0, st>>>(G + 1, goff64, goff);
  MG_TRY(B.alloc(&gsrc, S));
  k_group_fill<<<grid_of(32 * G), 256, 0, st>>>(G, U, perm, useg, src, uslot, umirror, goff, gsrc, gslot, gmirror);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaStreamSynchronize(st));
  p->d_goff = goff;
  p->d_uslot = gslot;
  p->d_umirror = gmirror;
  p->d_src = gsrc;
  p->n_upper = U;
  p->n_groups = G;
  p->n_diag = ndiag;
  p->n_slot_contrib = C;
  p->n_src = S;
  for (void* q : {(void*)goff, (void*)gslot, (void*)gmirror, (void*)gsrc}) B.keep(q);
  return MG_OK;
}


// ------------------------------------------------------------- block map --
// The one-pass P1 assembly's layout (see mg_plan::d_bgrp) from the slot map's
// per-entry source lists (p nu + u, ascending p):
//   1. runs per upper entry (block changes along its sources) and their prefix;
//      the shared entries (more than one run) and their prefix;
//   2. one record per run, radix-sorted (stable) by (block, longest first):
//      runs of equal length (or 63 and more) in CSR order;
//   3. groups of 32 runs per block, each sized by its longest run;
//   4. the shared entries sorted (stable) by run count, most first, in groups
//      of 32 sized by their most runs: the partial-sum slots, which fix each
//      run's output;
//   5. one thread per (group, lane): the local sources and the output.
mg_status build_block_map(mg_plan* p, int64_t U, const int32_t* useg, const int32_t* uslot, const int32_t* umirror,
                          const uint32_t* src, cudaStream_t st)
{
  const int nu = nunique(p->mesh->order), be = elems_per_block(p->mesh->order);
  if (be * nu >= UINT16_MAX) return set_error(MG_ERR_SIZE, "block map: a block's entries above 16 bits");
  const int64_t E = p->mesh->n_elem;
  const int64_t nblk = std::max<int64_t>(1, (E + be - 1) / be);
  const int64_t nseg = nblk;
  if (64 * nblk >= UINT32_MAX / 2) return set_error(MG_ERR_SIZE, "block map: too many element blocks");
  SchedBuffers B;
  int32_t *nrun, *shared, *rfirst, *sidx;
  MG_TRY(B.alloc(&nrun, U + 1));
  MG_TRY(B.alloc(&shared, U + 1));
  MG_TRY(B.alloc(&rfirst, U + 1));
  MG_TRY(B.alloc(&sidx, U + 1));
  k_run_count<<<grid_of(U + 1), 256, 0, st>>>(U, nu, be, useg, src, nrun, shared);
  MG_CUDA(cudaGetLastError());
  MG_TRY(exclusive_scan(B, nrun, rfirst, U + 1, st));
  MG_TRY(exclusive_scan(B, shared, sidx, U + 1, st));
  int32_t R = 0, S = 0;
  MG_TRY(read_back(&R, rfirst + U, st));
  MG_TRY(read_back(&S, sidx + U, st));
  // ---- runs, sorted by (block, length); the sort is stable, so CSR order within
  uint32_t *rkey, *skey, *rid, *perm;
  int32_t *rt, *rj, *rstart, *rlen;
  MG_TRY(B.alloc(&rkey, R));
  MG_TRY(B.alloc(&skey, R));
  MG_TRY(B.alloc(&rid, R));
  MG_TRY(B.alloc(&perm, R));
  MG_TRY(B.alloc(&rt, R));
  MG_TRY(B.alloc(&rj, R));
  MG_TRY(B.alloc(&rstart, R));
  MG_TRY(B.alloc(&rlen, R));
  if (U > 0)
    k_run_emit<<<grid_of(U), 256, 0, st>>>(U, nu, be, useg, src, rfirst, rkey, rid, rt, rj, rstart, rlen);
  int kbits = 1;
  while ((1ll << kbits) <= 64 * nblk) ++kbits;
  size_t tb = 0;
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, rkey, skey, rid, perm, (int)R, 0, kbits, st));
  unsigned char* tmp;
  MG_TRY(B.alloc(&tmp, (int64_t)std::max(tb, (size_t)1)));
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, rkey, skey, rid, perm, (int)R, 0, kbits, st));
  // ---- groups of 32 runs per block
  int32_t *seg_ptr, *ng, *seg_g;
  MG_TRY(B.alloc(&seg_ptr, nseg + 1));
  MG_TRY(B.alloc(&ng, nseg + 1));
  MG_TRY(B.alloc(&seg_g, nseg + 1));
  k_run_starts<<<grid_of((int64_t)R + 1), 256, 0, st>>>(R, skey, nseg, seg_ptr, 6);
  k_seg_groups<<<grid_of(nseg + 1), 256, 0, st>>>(nseg, seg_ptr, ng);
  MG_CUDA(cudaGetLastError());
  MG_TRY(exclusive_scan(B, ng, seg_g, nseg + 1, st));
  int32_t G = 0;
  MG_TRY(read_back(&G, seg_g + nseg, st));
  int32_t *grun0, *gcnt, *glen, *bgoff;
  MG_TRY(B.alloc(&grun0, G));
  MG_TRY(B.alloc(&gcnt, G));
  MG_TRY(B.alloc(&glen, (int64_t)G + 1));
  k_seg_fill<<<grid_of(nseg), 256, 0, st>>>(nseg, seg_ptr, seg_g, grun0, gcnt);
  k_bgroup_len<<<grid_of((int64_t)G + 1), 256, 0, st>>>(G, grun0, gcnt, perm, rlen, glen);
  MG_CUDA(cudaGetLastError());
  int64_t nsrc = 0;
  MG_TRY(narrow_offsets(B, glen, G, &bgoff, &nsrc, "block map: padded sources", st));
  // ---- shared entries (most runs first) and their partial-sum slots
  const int64_t G3 = ((int64_t)S + 31) / 32;
  int32_t *sh_csr, *sh_t, *srank, *slen, *sgoff;
  uint32_t *shk, *shk2;
  int2* sout;
  MG_TRY(B.alloc(&sh_csr, S));
  MG_TRY(B.alloc(&sh_t, S));
  MG_TRY(B.alloc(&srank, U));
  MG_TRY(B.alloc(&shk, S));
  MG_TRY(B.alloc(&shk2, S));
  MG_TRY(B.alloc(&slen, G3 + 1));
  MG_TRY(B.alloc(&sout, 32 * G3));
  if (U > 0) k_shared_list<<<grid_of(U), 256, 0, st>>>(U, shared, sidx, sh_csr);
  if (S > 0) k_shared_keys<<<grid_of(S), 256, 0, st>>>(S, sh_csr, nrun, shk);
  size_t tb5 = 0;
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb5, shk, shk2, sh_csr, sh_t, (int)S, 0, 6, st));
  unsigned char* tmp5;
  MG_TRY(B.alloc(&tmp5, (int64_t)std::max(tb5, (size_t)1)));
  MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp5, tb5, shk, shk2, sh_csr, sh_t, (int)S, 0, 6, st));
  if (S > 0) k_shared_rank<<<grid_of(S), 256, 0, st>>>(S, sh_t, srank);
  k_sgroup_len<<<grid_of(G3 + 1), 256, 0, st>>>(G3, S, sh_t, nrun, slen);
  MG_CUDA(cudaGetLastError());
  int64_t Q = 0;
  MG_TRY(narrow_offsets(B, slen, G3, &sgoff, &Q, "block map: partial sums", st));
  if (G3 > 0) k_sgroup_out<<<grid_of(32 * G3), 256, 0, st>>>(G3, S, sh_t, uslot, umirror, sout);
  // ---- local sources and outputs
  uint16_t* bsrc;
  int2* bout;
  int32_t *bgrp, *bsrc0;
  void* partial;
  MG_TRY(B.alloc(&bsrc, nsrc));
  MG_TRY(B.alloc(&bout, 32 * (int64_t)G));
  MG_TRY(B.alloc(&bgrp, nblk + 1));
  MG_TRY(B.alloc(&bsrc0, nblk + 1));
  MG_TRY(B.alloc(reinterpret_cast<double**>(&partial), Q));
  MG_CUDA(cudaMemsetAsync(partial, 0, sizeof(double) * (size_t)std::max<int64_t>(Q, 1), st));
  if (G > 0)
    k_bfill<<<grid_of(32 * (int64_t)G), 256, 0, st>>>(G, nu, be, grun0, gcnt, perm, skey, rt, rj, rstart, rlen, src, uslot,
                                                      umirror, nrun, srank, sgoff, bgoff, bsrc, bout);
  k_bgrp<<<grid_of(nblk + 1), 256, 0, st>>>(nblk, seg_g, bgoff, bgrp, bsrc0);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaStreamSynchronize(st));
  p->d_bgrp = bgrp;
  p->d_bsrc0 = bsrc0;
  p->d_bgoff = bgoff;
  p->d_bsrc = bsrc;
  p->d_bout = bout;
  p->d_sgoff = sgoff;
  p->d_sout = sout;
  p->d_partial = partial;
  p->n_blocks = nblk;
  p->n_bgroups = G;
  p->n_bsrc = nsrc;
  p->n_runs = R;
  p->n_shared = S;
  p->n_sgroups = G3;
  p->n_partial = Q;
  for (void* q : {(void*)bgrp, (void*)bsrc0, (void*)bgoff, (void*)bsrc, (void*)bout, (void*)sgoff, (void*)sout,
                  partial})
    B.keep(q);
  return MG_OK;
}

// The plan's device state from its device pattern: the Morton element order,
// the dofs in that order, the diagonal entries and 16-bit column offsets, the
// status counters and the slot map -- the arrays plan_device makes for a
// host-built plan, from the same rules.
mg_status build_plan_device(mg_plan* p, cudaStream_t st)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = p->ndof, N = m->n_nodes;
  if (!p->d_rowptr || !p->d_colind) return set_error(MG_ERR_INVALID_ARG, "device plan: pattern not on the device");
  if (nd >= INT32_MAX / 2 || E * nb >= INT32_MAX) return set_error(MG_ERR_SIZE, "device plan: sizes above 2^30");
  MG_TRY(mesh_device(m));
  SchedBuffers B;
  // ---- elements along the Morton curve of their centroids
  Box bx;
  for (int k = 0; k < 3; ++k) bx.lo[k] = INFINITY, bx.hi[k] = -INFINITY;
  for (int64_t i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) {
      bx.lo[k] = std::min(bx.lo[k], m->xyz[3 * i + k]);
      bx.hi[k] = std::max(bx.hi[k], m->xyz[3 * i + k]);
    }
  uint64_t *ka, *kb;
  int32_t *ia, *d_elem_order;
  MG_TRY(B.alloc(&ka, E));
  MG_TRY(B.alloc(&kb, E));
  MG_TRY(B.alloc(&ia, E));
  MG_TRY(B.alloc(&d_elem_order, E));
  size_t tb = 0;
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, ka, kb, ia, d_elem_order, (int)E, 0, 64, st));
  unsigned char* tmp;
  MG_TRY(B.alloc(&tmp, (int64_t)tb));
  if (E > 0) {
    k_elem_keys<<<grid_of(E), 256, 0, st>>>(E, m->d_conn, m->d_xyz, bx, ka, ia);
    MG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, ka, kb, ia, d_elem_order, (int)E, 0, 64, st));
  }
  int32_t* d_dm;
  MG_TRY(B.alloc(&d_dm, E * nb));
  if (E > 0) k_dofs_morton<<<grid_of(E * nb), 256, 0, st>>>(E, nb, d_elem_order, m->d_dofs, d_dm);
  // ---- diagonal entries, 16-bit column offsets
  int32_t* d_diag;
  int16_t* d_coloff;
  int* d_fits;
  MG_TRY(B.alloc(&d_diag, nd));
  MG_TRY(B.alloc(&d_coloff, p->nnz));
  MG_TRY(B.alloc(&d_fits, 1));
  const int one = 1;
  MG_CUDA(cudaMemcpyAsync(d_fits, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  if (nd > 0) k_diag_coloff<<<grid_of(nd), 256, 0, st>>>(nd, p->d_rowptr, p->d_colind, d_diag, d_coloff, d_fits);
  MG_CUDA(cudaGetLastError());
  int fits = 0;
  MG_CUDA(cudaMemcpyAsync(&fits, d_fits, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_TRY(download(p->h_elem_order, d_elem_order, E, st));
  uint32_t* d_counters;
  MG_TRY(upload_to(B, &d_counters, std::vector<uint32_t>(8, 0u), st));
  MG_CUDA(cudaStreamSynchronize(st));
  if (!p->h_pinned) MG_CUDA(cudaMallocHost(&p->h_pinned, 64 * sizeof(double)));
  p->d_diag = d_diag;
  p->d_coloff = (fits && p->nnz > 0) ? d_coloff : nullptr;
  p->d_elem_order = d_elem_order;
  p->d_dofs_morton = d_dm;
  p->d_counters = d_counters;
  for (void* q : {(void*)d_diag, (void*)d_elem_order, (void*)d_dm, (void*)d_counters}) B.keep(q);
  if (p->d_coloff) B.keep(d_coloff);
  MG_TRY(build_slot_map(p, st));
  p->on_device = true;
  return MG_OK;
}

}  // namespace mg
