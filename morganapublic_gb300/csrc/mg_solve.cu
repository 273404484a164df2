// CSR SpMV and conjugate-gradient solvers for sm_103a.
//
// SpMV: FP64 one thread per row (the FP64 pipe, not HBM, is the narrow
// resource on GB300); FP32 a group of G lanes per row (G from the mean row
// length), values and column indices read coalesced, x gathered through the
// read-only path, the row sum reduced with xor shuffles in a fixed tree --
// deterministic.
//
// CG: the reference hands the assembled Epetra operator to Belos BlockCG
// (src/morganaTrilinos/belosBlockCG.hpp:46-82 in morganaPublic); here every
// iteration is three kernels whose scalars (alpha, beta, r.z, r.r, a done flag)
// live in device memory:
//   K1  q = A p and per-CTA partials of p.q; the last CTA to finish (integer
//       ticket) sums the partials in a fixed order and sets alpha = rz / pq;
//   K2  x += alpha p, r -= alpha q, z = D^-1 r, partials of r.z and r.r; the last
//       CTA forms beta, rz, rr and raises `done` when ||r|| <= tol ||b||;
//   K3  p = z + beta p.
// Once `done` is set the remaining kernels return at entry, so a CUDA graph of
// several iterations can be replayed without a host round trip per iteration.
// Kernels are launched with programmatic dependent launch: a kernel's launch and
// prologue overlap the tail of the one before, and it waits (griddepcontrol)
// before touching memory that kernel wrote.
// Dot products accumulate in FP64 in both precisions; the order of every
// floating-point sum is fixed, so a solve is bitwise reproducible.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "mg_ff.cuh"
#include "mg_internal.h"

namespace mg {

constexpr int kSolveThreads = 256;
constexpr int kMaxSolveBlocks = 2048;  // bound of the per-CTA partial arrays

// Programmatic dependent launch: wait for the preceding kernel's memory (a no-op
// when there is no programmatic dependency), and let the next kernel be
// scheduled once every CTA of this one has started.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st,
                            Args&&... args)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args&&... args)
{
  return launch_k(true, kernel, grid, block, st, std::forward<Args>(args)...);
}

struct CgScalars {
  double rz, alpha, beta, rr, bb, tol2, pq, rz_prev;
  double rr_anchor, delta2, pad[2];  // reliable updates: r.r at the last anchor, trigger ratio^2 (0 = off)
  int32_t done, iter, maxit, pad2;
  uint32_t ticket[4];
};
// done: 0 running, 1 converged (recursive residual), 2 breakdown (p.Ap <= 0),
// 3 maxit, 5 pause for a reliable update

// ------------------------------------------------------------ launch shape --
// GB300 issues FP64 at ~1/60 of its FP32 rate, below the rate at which HBM
// delivers doubles, so FP64 kernels are shaped to issue as few FP64 operations
// per entry as possible: one thread per CSR row (one FMA per entry, no
// shuffle-adds) with 16 entries loaded per pass and two accumulators, and
// several vector entries per thread (the block reduction tree is paid once per
// thread).  FP32 kernels use groups of 2+ lanes x 8 entries per row and more threads.
// SMs of the current device (cached per device; racing first calls store the
// same value)
static int sm_count()
{
  static std::atomic<int> cached[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int sms = cached[dev].load(std::memory_order_relaxed);
  if (sms <= 0) {
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    cached[dev].store(sms, std::memory_order_relaxed);
  }
  return sms;
}

template <typename V> constexpr int kEntriesPerLane = sizeof(V) == 8 ? 16 : 8;

// FP64 row shape.  GB300 issues 2 FP64 FMA lanes per SM per clock, about as many
// products as HBM delivers matrix entries, and a warp instruction occupies the
// FP64 pipe whatever its active lanes: every lane of a warp issues the FMAs of
// the passes its longest row needs.  The FP64 kernels therefore prefer one
// thread per row (no shuffle-adds) with 15 entries per pass: interior P1 rows
// have 15 entries, one pass; P2 rows (19, 27 and 65 entries) take 2, 2 and 5.
// The standalone SpMV keeps two lanes per row for rows above 16 entries on
// average: there single-lane loads cost more L1 throughput than the FMAs they
// save (measured on GB300 at P2 48^3: 101 us against 99 us with two lanes of
// 16).  Two lanes of 14 (28 entries per pass: P2 rows of 19 and 27 in one pass,
// 65 in three; ~1.38 FMA slots per entry against ~1.56 with 16) measured 90.8
// against 99.0 us there.
constexpr int kF64Entries = 15;
constexpr int kF64PairEntries = 14;

// Lanes per row of the standalone SpMV: FP64 one up to 16 entries on average
// (P1), two above (P2); FP32 the smallest group of at least 2 lanes whose pass
// covers the mean row length (measured on GB300 at P1 128^3 and P2 48^3).
template <typename V>
static int row_group(int64_t rows, int64_t nnz)
{
  const double mean = rows > 0 ? (double)nnz / (double)rows : 1.0;
  if (sizeof(V) == 8) return mean > 16.0 ? 2 : 1;
  const int U = kEntriesPerLane<V>;
  for (int g = 2; g < 32; g *= 2)
    if (mean <= g * U) return g;
  return 32;
}
template <typename V>
static int row_group(const mg_plan* p)
{
  return row_group<V>(p->ndof, p->nnz);
}

// CTAs covering every row once (G lanes per row), for the standalone SpMV.
static int spmv_full_grid(int64_t rows, int G)
{
  return (int)std::max<int64_t>(1, std::min<int64_t>((rows * G + kSolveThreads - 1) / kSolveThreads, INT32_MAX));
}

// CTAs of a row kernel with G lanes per row, at most `per_sm` per SM.
static int row_blocks(int64_t rows, int G, int per_sm)
{
  const int64_t need = (rows * G + kSolveThreads - 1) / kSolveThreads;
  const int cap = per_sm * sm_count();
  return (int)std::max<int64_t>(1, std::min<int64_t>({need, (int64_t)cap, (int64_t)kMaxSolveBlocks}));
}
static int row_blocks(const mg_plan* p, int G, int per_sm)
{
  return row_blocks(p->ndof, G, per_sm);
}
template <typename V>
static int row_blocks(const mg_plan* p, int G)
{
  return row_blocks(p, G, 8);
}

// Shape of the CG kernels: FP64 one thread per row, 15 entries per pass (the
// FP64 row shape above; measured on GB300 against two or four lanes of 8: 151
// against 159 us per iteration at P1 128^3, 136 against 142 us at P2 48^3);
// FP32 rows by 2 lanes x 8 entries (more lanes for longer rows).  FP64 at most
// 4 CTAs per SM (fewer partials for the last CTA to sum) and launched without
// programmatic dependent launch (it slowed the FP64 iteration); FP32 up to 8
// CTAs per SM, with programmatic dependent launch.
template <typename V> struct CgShape {
  static constexpr int U = sizeof(V) == 8 ? kF64Entries : 8;
  static constexpr bool pdl = sizeof(V) == 4;
  static int group(const mg_plan* p)
  {
    if (sizeof(V) == 8) return 1;
    const double mean = p->ndof > 0 ? (double)p->nnz / (double)p->ndof : 1.0;
    for (int g = 2; g < 32; g *= 2)
      if (mean <= g * U) return g;
    return 32;
  }
  static int blocks(const mg_plan* p, int G) { return row_blocks(p, G, sizeof(V) == 8 ? 4 : 8); }
};

template <typename V>
static int vec_blocks(int64_t n)
{
  const int64_t need = (n + kSolveThreads - 1) / kSolveThreads;
  const int cap = (sizeof(V) == 8 ? 2 : 4) * sm_count();
  return (int)std::max<int64_t>(1, std::min<int64_t>({need, (int64_t)cap, (int64_t)kMaxSolveBlocks}));
}

template <int G>
__device__ __forceinline__ unsigned group_mask()
{
  if constexpr (G == 32) {
    return 0xffffffffu;
  } else {
    const unsigned lane = threadIdx.x & 31u;
    return ((1u << G) - 1u) << (lane & ~(unsigned)(G - 1));
  }
}

// Dot product of one CSR row with x by a group of G lanes.  Each pass issues
// U independent loads of (column, value) per lane before any gather of x, so
// every lane keeps U requests in flight; the G partial sums are combined by xor
// shuffles in a fixed order.
// Entries u of a pass alternate between two accumulators (halving the chain of
// dependent FMAs), added at the end.
// Column of entry s of `row`: int32 columns, or 16-bit offsets col - row (the
// plan's compressed index stream).
template <typename I>
__device__ __forceinline__ int column(const I* __restrict__ ci, int s, int64_t row)
{
  if constexpr (sizeof(I) == 2) return (int)row + (int)__ldg(ci + s);
  else return __ldg(ci + s);
}

template <typename V, int G, int U = kEntriesPerLane<V>, typename I = int32_t>
__device__ __forceinline__ V row_dot(int64_t row, const int32_t* __restrict__ rp, const I* __restrict__ ci,
                                     const V* __restrict__ val, const V* __restrict__ x)
{
  const int lane = threadIdx.x & (G - 1);
  const int s0 = __ldg(rp + row), s1 = __ldg(rp + row + 1);
  V sa = V(0), sb = V(0);
  for (int base = s0 + lane; base < s1; base += G * U) {
    int c[U];
    V v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int s = base + u * G;
      c[u] = s < s1 ? column<I>(ci, s, row) : -1;
      v[u] = s < s1 ? __ldg(val + s) : V(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const V xv = c[u] >= 0 ? __ldg(x + c[u]) : V(0);
      if (u & 1) sb = fma(v[u], xv, sb);
      else sa = fma(v[u], xv, sa);
    }
  }
  V sum = sa + sb;
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) sum += __shfl_xor_sync(group_mask<G>(), sum, off, G);
  return sum;
}

// Dot-product accumulation: FP64 for FP64 vectors; for FP32 vectors a
// double-word (float pair) sum of exact float products on the FP32 pipes, as
// accurate as FP64 here and free of FP64 operations.
template <typename V> struct Dot;
template <> struct Dot<double> {
  using A = double;
  __device__ static A zero() { return 0.0; }
  __device__ static void mac(A& s, double a, double b) { s = __fma_rn(a, b, s); }
  __device__ static A add(A a, A b) { return a + b; }
  __device__ static A shfl(A v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
  __device__ static double to_double(A v) { return v; }
};
template <> struct Dot<float> {
  using A = ff;
  __device__ static A zero() { return ff{0.0f, 0.0f}; }
  __device__ static void mac(A& s, float a, float b) { s = ff_add_s(s, two_prod(a, b)); }
  __device__ static A add(A a, A b) { return ff_add_s(a, b); }
  __device__ static A shfl(A v, int off)
  {
    return ff{__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off)};
  }
  __device__ static double to_double(A v) { return (double)v.hi + (double)v.lo; }
};

// Block-wide sum in a fixed tree; the result (as double) is valid in thread 0.
template <typename V>
__device__ __forceinline__ double block_sum(typename Dot<V>::A v, typename Dot<V>::A* sh)
{
  using D = Dot<V>;
  const int tid = threadIdx.x;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = D::add(v, D::shfl(v, off));
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  double out = 0.0;
  if (tid < 32) {
    v = tid < (kSolveThreads / 32) ? sh[tid] : D::zero();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = D::add(v, D::shfl(v, off));
    if (tid == 0) out = D::to_double(v);
  }
  __syncthreads();
  return out;
}

// NV block-wide sums at once (each value the same fixed tree as block_sum, so
// the results are those of NV separate calls, with two barriers instead of 2 NV);
// sh holds NV * 32 values.  Valid in thread 0.
template <typename V, int NV>
__device__ __forceinline__ void block_sum_n(typename Dot<V>::A (&v)[NV], typename Dot<V>::A* sh, double (&out)[NV])
{
  using D = Dot<V>;
  const int tid = threadIdx.x;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = D::add(v[k], D::shfl(v[k], off));
  if ((tid & 31) == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + (tid >> 5)] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) out[k] = 0.0;
  if (tid < 32) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = tid < (kSolveThreads / 32) ? sh[k * 32 + tid] : D::zero();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) v[k] = D::add(v[k], D::shfl(v[k], off));
    if (tid == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) out[k] = D::to_double(v[k]);
  }
  __syncthreads();
}

// Sum of partials[0..n) in a fixed order by one CTA (valid in thread 0).
__device__ __forceinline__ double reduce_partials(const double* partials, int n, double* sh)
{
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kSolveThreads) v += partials[i];
  return block_sum<double>(v, sh);
}

// NV arrays of partials (partials[k * n + i]) reduced together, each in the
// order of reduce_partials; sh holds NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void reduce_partials_n(const double* partials, int n, double* sh, double (&out)[NV])
{
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int i = threadIdx.x; i < n; i += kSolveThreads)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += partials[k * n + i];
  block_sum_n<double, NV>(v, sh, out);
}

// Last-CTA detection: returns true in the single CTA that finishes last.
__device__ __forceinline__ bool last_block(uint32_t* ticket)
{
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const uint32_t t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

template <typename V, int G, int U, typename I>
__global__ void __launch_bounds__(kSolveThreads) k_spmv(int64_t n, const int32_t* __restrict__ rp,
                                                        const I* __restrict__ ci, const V* __restrict__ val,
                                                        const V* __restrict__ x, V* __restrict__ y)
{
  pdl_wait();
  pdl_trigger();
  const int64_t groups = (int64_t)gridDim.x * (kSolveThreads / G);
  for (int64_t row = (blockIdx.x * (int64_t)kSolveThreads + threadIdx.x) / G; row < n; row += groups) {
    const V s = row_dot<V, G, U, I>(row, rp, ci, val, x);
    if ((threadIdx.x & (G - 1)) == 0) y[row] = s;
  }
}

// K1: q = A p, alpha = rz / (p . q)
template <typename V, int G, typename I>
__global__ void __launch_bounds__(kSolveThreads) k_cg_spmv(int64_t n, const int32_t* __restrict__ rp,
                                                           const I* __restrict__ ci, const V* __restrict__ val,
                                                           const V* __restrict__ p, V* __restrict__ q,
                                                           double* partials, CgScalars* s)
{
  using D = Dot<V>;
  __shared__ typename D::A sh[32];
  __shared__ double shd[32];
  pdl_wait();
  pdl_trigger();
  if (s->done) return;
  const int64_t groups = (int64_t)gridDim.x * (kSolveThreads / G);
  typename D::A acc = D::zero();
  for (int64_t row = (blockIdx.x * (int64_t)kSolveThreads + threadIdx.x) / G; row < n; row += groups) {
    const V v = row_dot<V, G, CgShape<V>::U, I>(row, rp, ci, val, p);
    if ((threadIdx.x & (G - 1)) == 0) {
      q[row] = v;
      D::mac(acc, p[row], v);
    }
  }
  const double b = block_sum<V>(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
  if (last_block(&s->ticket[0])) {
    const double pq = reduce_partials(partials, gridDim.x, shd);
    if (threadIdx.x == 0) {
      s->pq = pq;
      s->alpha = s->rz / pq;
      if (!(pq > 0.0) || !isfinite(s->alpha)) s->done = 2;  // breakdown: A not SPD on the Krylov space
      s->ticket[0] = 0;
    }
  }
}

// K2: x += alpha p; r -= alpha q; z = D^-1 r; rz, rr, beta, convergence
template <typename V>
__global__ void __launch_bounds__(kSolveThreads) k_cg_update(int64_t n, V* __restrict__ x, V* __restrict__ r,
                                                             V* __restrict__ z, const V* __restrict__ p,
                                                             const V* __restrict__ q, const V* __restrict__ dinv,
                                                             double* partials, CgScalars* s)
{
  using D = Dot<V>;
  __shared__ typename D::A sh[2 * 32];
  __shared__ double shd[2 * 32];
  pdl_wait();
  pdl_trigger();
  if (s->done) return;
  const V alpha = (V)s->alpha;
  typename D::A prz = D::zero(), prr = D::zero();
#pragma unroll 4
  for (int64_t i = blockIdx.x * (int64_t)kSolveThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kSolveThreads) {
    x[i] += alpha * p[i];
    const V ri = r[i] - alpha * q[i];
    r[i] = ri;
    const V zi = dinv[i] * ri;
    z[i] = zi;
    D::mac(prz, ri, zi);
    D::mac(prr, ri, ri);
  }
  typename D::A acc2[2] = {prz, prr};
  double bl[2];
  block_sum_n<V, 2>(acc2, sh, bl);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = bl[0];
    partials[gridDim.x + blockIdx.x] = bl[1];
  }
  if (last_block(&s->ticket[1])) {
    double tot[2];
    reduce_partials_n<2>(partials, gridDim.x, shd, tot);
    const double rz = tot[0], rr = tot[1];
    if (threadIdx.x == 0) {
      s->rz_prev = s->rz;
      s->beta = rz / s->rz;
      s->rz = rz;
      s->rr = rr;
      s->iter += 1;
      if (rr <= s->tol2 * s->bb) s->done = 1;
      else if (s->iter >= s->maxit) s->done = 3;
      else if (rr <= s->delta2 * s->rr_anchor) s->done = 5;  // K3 is skipped: the host re-anchors first
      s->ticket[1] = 0;
    }
  }
}

// K3: p = z + beta p
template <typename V>
__global__ void __launch_bounds__(kSolveThreads) k_cg_dir(int64_t n, const V* __restrict__ z, V* __restrict__ p,
                                                          const CgScalars* s)
{
  pdl_wait();
  pdl_trigger();
  if (s->done) return;
  const V beta = (V)s->beta;
#pragma unroll 4
  for (int64_t i = blockIdx.x * (int64_t)kSolveThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kSolveThreads)
    p[i] = z[i] + beta * p[i];
}

// Start of a solve: r = b - A x (or r = b when x is zero), z = D^-1 r, p = z,
// D^-1 from the diagonal, partials of r.z, r.r, b.b.
template <typename V, int G>
__global__ void __launch_bounds__(kSolveThreads) k_cg_start(int64_t n, const int32_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci, const V* __restrict__ val,
                                                            const int32_t* __restrict__ diag, const V* __restrict__ b,
                                                            const V* __restrict__ x, int zero_x, int jacobi,
                                                            V* __restrict__ r, V* __restrict__ z, V* __restrict__ p,
                                                            V* __restrict__ dinv, double* partials, CgScalars* s)
{
  using D = Dot<V>;
  __shared__ typename D::A sh[3 * 32];
  __shared__ double shd[3 * 32];
  const int64_t groups = (int64_t)gridDim.x * (kSolveThreads / G);
  typename D::A prz = D::zero(), prr = D::zero(), pbb = D::zero();
  for (int64_t row = (blockIdx.x * (int64_t)kSolveThreads + threadIdx.x) / G; row < n; row += groups) {
    V ax = V(0);
    if (!zero_x) ax = row_dot<V, G, CgShape<V>::U>(row, rp, ci, val, x);
    if ((threadIdx.x & (G - 1)) == 0) {
      const V dv = val[diag[row]];
      const V di = (jacobi && dv != V(0)) ? V(1) / dv : V(1);
      const V ri = b[row] - ax;
      const V zi = di * ri;
      dinv[row] = di;
      r[row] = ri;
      z[row] = zi;
      p[row] = zi;
      D::mac(prz, ri, zi);
      D::mac(prr, ri, ri);
      D::mac(pbb, b[row], b[row]);
    }
  }
  typename D::A acc3[3] = {prz, prr, pbb};
  double bl[3];
  block_sum_n<V, 3>(acc3, sh, bl);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = bl[0];
    partials[gridDim.x + blockIdx.x] = bl[1];
    partials[2 * gridDim.x + blockIdx.x] = bl[2];
  }
  if (last_block(&s->ticket[2])) {
    double tot[3];
    reduce_partials_n<3>(partials, gridDim.x, shd, tot);
    const double rz = tot[0], rr = tot[1], bb = tot[2];
    if (threadIdx.x == 0) {
      s->rz = rz;
      s->rr = rr;
      s->bb = bb > 0.0 ? bb : 1.0;
      s->iter = 0;
      s->done = (rr <= s->tol2 * s->bb) ? 1 : 0;
      s->ticket[2] = 0;
    }
  }
}

// Refinement residual: r64 = b - A64 x, rr = r64 . r64 (last CTA); the scaled
// FP32 right-hand side r32 = r64 / ||r64|| is then written by k_scale_cast.
template <int G>
__global__ void __launch_bounds__(kSolveThreads) k_residual64(int64_t n, const int32_t* __restrict__ rp,
                                                              const int32_t* __restrict__ ci,
                                                              const double* __restrict__ val,
                                                              const double* __restrict__ b,
                                                              const double* __restrict__ x, double* __restrict__ r,
                                                              double* partials, CgScalars* s)
{
  __shared__ double sh[2 * 32];
  const int64_t groups = (int64_t)gridDim.x * (kSolveThreads / G);
  double prr = 0.0, pbb = 0.0;
  for (int64_t row = (blockIdx.x * (int64_t)kSolveThreads + threadIdx.x) / G; row < n; row += groups) {
    const double ax = row_dot<double, G, CgShape<double>::U>(row, rp, ci, val, x);
    if ((threadIdx.x & (G - 1)) == 0) {
      const double ri = b[row] - ax;
      r[row] = ri;
      prr = __fma_rn(ri, ri, prr);
      pbb = __fma_rn(b[row], b[row], pbb);
    }
  }
  double acc2[2] = {prr, pbb}, bl[2];
  block_sum_n<double, 2>(acc2, sh, bl);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = bl[0];
    partials[gridDim.x + blockIdx.x] = bl[1];
  }
  if (last_block(&s->ticket[3])) {
    double tot[2];
    reduce_partials_n<2>(partials, gridDim.x, sh, tot);
    const double rr = tot[0], bb = tot[1];
    if (threadIdx.x == 0) {
      s->rr = rr;
      s->bb = bb > 0.0 ? bb : 1.0;
      s->ticket[3] = 0;
    }
  }
}

__global__ void k_scale_cast(int64_t n, const double* r, double scale, float* r32, float* d32)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    r32[i] = (float)(r[i] * scale);
    d32[i] = 0.0f;
  }
}

// Reliable update, part 1: x64 += x32, x32 = 0.
__global__ void k_anchor_x(int64_t n, double* __restrict__ x, float* __restrict__ x32)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)x32[i];
    x32[i] = 0.0f;
  }
}

// Reliable update, part 2 (after r64 = b - A64 x): r32 = r64, z32 = D^-1 r32,
// r.z and r.r of the replaced residual; the last CTA forms beta with the r.z
// of the iteration that paused, re-anchors and resumes (K3 then runs).
__global__ void __launch_bounds__(kSolveThreads) k_anchor_r(int64_t n, const double* __restrict__ r64,
                                                            float* __restrict__ r, float* __restrict__ z,
                                                            const float* __restrict__ dinv, double* partials,
                                                            CgScalars* s)
{
  using D = Dot<float>;
  __shared__ D::A sh[2 * 32];
  __shared__ double shd[2 * 32];
  D::A prz = D::zero(), prr = D::zero();
  for (int64_t i = blockIdx.x * (int64_t)kSolveThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kSolveThreads) {
    const float ri = (float)r64[i];
    const float zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    D::mac(prz, ri, zi);
    D::mac(prr, ri, ri);
  }
  D::A acc2[2] = {prz, prr};
  double bl[2];
  block_sum_n<float, 2>(acc2, sh, bl);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = bl[0];
    partials[gridDim.x + blockIdx.x] = bl[1];
  }
  if (last_block(&s->ticket[1])) {
    double tot[2];
    reduce_partials_n<2>(partials, gridDim.x, shd, tot);
    const double rz = tot[0], rr = tot[1];
    if (threadIdx.x == 0) {
      s->beta = rz / s->rz_prev;
      s->rz = rz;
      s->rr = rr;
      s->rr_anchor = rr;
      s->done = 0;
      s->ticket[1] = 0;
    }
  }
}

#define MG_DISPATCH_G(G, ...)                                \
  switch (G) {                                               \
    case 32: { constexpr int g = 32; __VA_ARGS__; } break;   \
    case 16: { constexpr int g = 16; __VA_ARGS__; } break;   \
    case 8: { constexpr int g = 8; __VA_ARGS__; } break;     \
    case 4: { constexpr int g = 4; __VA_ARGS__; } break;     \
    case 2: { constexpr int g = 2; __VA_ARGS__; } break;     \
    default: { constexpr int g = 1; __VA_ARGS__; } break;    \
  }

mg_status launch_spmv(mg_plan* p, int prec, const void* vals, const void* x, void* y, cudaStream_t st)
{
  if (!prec_valid(prec)) return set_error(MG_ERR_INVALID_ARG, "bad precision");
  if (p->ndof == 0) return MG_OK;
  if (!vals || !x || !y) return set_error(MG_ERR_INVALID_ARG, "mg_spmv: null argument");
  MG_TRY(plan_device(p));
  if (prec_is_f64(prec)) {
    // FP64: one thread per row, a CTA for every 256 rows, no grid-stride loop
    // (measured on GB300 at P1 128^3: 84.7 us against 88.7 us with 8 CTAs per SM
    // and a grid-stride loop)
    const int G = row_group<double>(p), nb = spmv_full_grid(p->ndof, G);
    const double *v = (const double*)vals, *xx = (const double*)x;
    double* yy = (double*)y;
    const int32_t* rp = p->d_rowptr;
    const int64_t n = p->ndof;
    if (p->d_coloff) {
      const int16_t* c = p->d_coloff;
      if (G == 1) launch_pdl(k_spmv<double, 1, kF64Entries, int16_t>, nb, kSolveThreads, st, n, rp, c, v, xx, yy);
      else launch_pdl(k_spmv<double, 2, kF64PairEntries, int16_t>, nb, kSolveThreads, st, n, rp, c, v, xx, yy);
    } else {
      const int32_t* c = p->d_colind;
      if (G == 1) launch_pdl(k_spmv<double, 1, kF64Entries, int32_t>, nb, kSolveThreads, st, n, rp, c, v, xx, yy);
      else launch_pdl(k_spmv<double, 2, kF64PairEntries, int32_t>, nb, kSolveThreads, st, n, rp, c, v, xx, yy);
    }
  } else {
    const int G = row_group<float>(p), nb = row_blocks<float>(p, G);
    if (p->d_coloff) {
      MG_DISPATCH_G(G, (launch_pdl(k_spmv<float, g, kEntriesPerLane<float>, int16_t>, nb, kSolveThreads, st, p->ndof,
                                   (const int32_t*)p->d_rowptr, (const int16_t*)p->d_coloff, (const float*)vals,
                                   (const float*)x, (float*)y)));
    } else {
      MG_DISPATCH_G(G, (launch_pdl(k_spmv<float, g, kEntriesPerLane<float>, int32_t>, nb, kSolveThreads, st, p->ndof,
                                   (const int32_t*)p->d_rowptr, (const int32_t*)p->d_colind, (const float*)vals,
                                   (const float*)x, (float*)y)));
    }
  }
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// y = A x for a CSR matrix of any shape: the standalone SpMV kernel with the
// lane group of the FP64 path, int32 columns.
mg_status launch_spmv_csr(int64_t rows, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                          const double* vals, const double* x, double* y, cudaStream_t st)
{
  if (rows == 0) return MG_OK;
  const int G = row_group<double>(rows, nnz), nb = row_blocks(rows, G, 8);
  if (G == 1)
    launch_pdl(k_spmv<double, 1, kF64Entries, int32_t>, nb, kSolveThreads, st, rows, rowptr, colind, vals, x, y);
  else
    launch_pdl(k_spmv<double, 2, kF64PairEntries, int32_t>, nb, kSolveThreads, st, rows, rowptr, colind, vals, x,
               y);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}


// Workspace of one CG run over vectors of type V.
template <typename V>
struct CgWork {
  V *r, *z, *p, *q, *dinv;
  double* partials;  // 3 * kMaxSolveBlocks
  CgScalars* s;
};

template <typename V>
static size_t cg_work_bytes(int64_t n)
{
  const size_t vec = ((size_t)n * sizeof(V) + 255) / 256 * 256;
  return 5 * vec + 3 * kMaxSolveBlocks * sizeof(double) + 256;
}

template <typename V>
static CgWork<V> cg_work_carve(void* base, int64_t n)
{
  char* c = (char*)base;
  const size_t vec = ((size_t)n * sizeof(V) + 255) / 256 * 256;
  CgWork<V> w;
  w.s = (CgScalars*)c;
  c += 256;
  w.partials = (double*)c;
  c += 3 * kMaxSolveBlocks * sizeof(double);
  w.r = (V*)c; c += vec;
  w.z = (V*)c; c += vec;
  w.p = (V*)c; c += vec;
  w.q = (V*)c; c += vec;
  w.dinv = (V*)c;
  return w;
}

// Smallest reliable-update trigger ratio of the mixed-precision CG.
constexpr double kMinAnchorRatio = 1e-3;

// Iterations per replay of the captured CG graph between two host checks.
constexpr int kGraphIters = 16;

// Runs CG on A (vals) from the state set up by k_cg_start until `done`.
template <typename V>
static mg_status cg_iterate(mg_plan* p, const V* vals, V* x, CgWork<V>& w, int G, int nb, int maxit,
                            cudaStream_t st, CgScalars* h_s)
{
  const int64_t n = p->ndof;
  const int vb = vec_blocks<V>(n);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool use_graph = true;
  cudaStreamCaptureStatus cs;
  MG_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone || st == nullptr) use_graph = false;  // no nested capture; legacy stream cannot capture
  constexpr bool pdl = CgShape<V>::pdl;
  auto body = [&]() {
    if (p->d_coloff) {
      MG_DISPATCH_G(G, (launch_k(pdl, k_cg_spmv<V, g, int16_t>, nb, kSolveThreads, st, n,
                                 (const int32_t*)p->d_rowptr, (const int16_t*)p->d_coloff, vals, (const V*)w.p, w.q,
                                 w.partials, w.s)));
    } else {
      MG_DISPATCH_G(G, (launch_k(pdl, k_cg_spmv<V, g, int32_t>, nb, kSolveThreads, st, n,
                                 (const int32_t*)p->d_rowptr, (const int32_t*)p->d_colind, vals, (const V*)w.p, w.q,
                                 w.partials, w.s)));
    }
    launch_k(pdl, k_cg_update<V>, vb, kSolveThreads, st, n, x, w.r, w.z, (const V*)w.p, (const V*)w.q,
             (const V*)w.dinv, w.partials, w.s);
    launch_k(pdl, k_cg_dir<V>, vb, kSolveThreads, st, n, (const V*)w.z, w.p, (const CgScalars*)w.s);
  };
  if (use_graph) {
    MG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kGraphIters; ++k) body();
    MG_CUDA(cudaStreamEndCapture(st, &graph));
    MG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  }
  mg_status status = MG_OK;
  for (int launched = 0;; launched += kGraphIters) {
    if (use_graph) {
      cudaError_t e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) { status = cuda_error(e, "cudaGraphLaunch"); break; }
    } else {
      for (int k = 0; k < kGraphIters; ++k) body();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) { status = cuda_error(e, "cg kernels"); break; }
    }
    cudaError_t e = cudaMemcpyAsync(h_s, w.s, sizeof(CgScalars), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { status = cuda_error(e, "cg scalars"); break; }
    if (h_s->done) break;
    if (launched + kGraphIters > maxit + kGraphIters) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  return status;
}

template <typename V>
static mg_status cg_start(mg_plan* p, const V* vals, const V* b, const V* x, int zero_x, int jacobi,
                          double tol, int maxit, CgWork<V>& w, int G, int nb, cudaStream_t st)
{
  CgScalars init{};
  init.tol2 = tol * tol;
  init.maxit = maxit;
  MG_CUDA(cudaMemcpyAsync(w.s, &init, sizeof(CgScalars), cudaMemcpyHostToDevice, st));
  const int64_t n = p->ndof;
  MG_DISPATCH_G(G, (k_cg_start<V, g><<<nb, kSolveThreads, 0, st>>>(n, p->d_rowptr, p->d_colind, vals, p->d_diag, b,
                                                                     x, zero_x, jacobi, w.r, w.z, w.p, w.dinv,
                                                                     w.partials, w.s)));
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// ||r|| / ||b|| from the squared norms; with b = 0 the absolute residual ||r||
// (0 when r = 0 as well), never NaN
static double rel_residual(double rr, double bb)
{
  if (rr == 0.0) return 0.0;
  return bb > 0.0 ? std::sqrt(rr / bb) : std::sqrt(rr);
}

// ------------------------------------------------- CG without allocation --
// Work space of mg_cg_solve_noalloc: a file-scope device array (16 MiB, 256-byte
// aligned), enough for the CG vectors of MG_CG_NOALLOC_MAX_NDOF dofs.  Host code
// must not use the symbol itself as a pointer: its device address is looked up
// once per device with cudaGetSymbolAddress.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static_assert(MG_CG_NOALLOC_MAX_NDOF > 0, "limit");

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

static mg_status noalloc_scratch(void** out)
{
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(MG_ERR_UNSUPPORTED, "device index above 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return MG_OK;
}

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_cg_solve_noalloc(mg_plan* p, const double* d_values, const double* d_b, double* d_x, double rtol,
                              int32_t maxit, int32_t precond, mg_cg_info* info, void* stream)
{
  NvtxRange nvtx_range("mg_cg_solve_noalloc");
  if (!p || !d_values || !d_b || !d_x) return set_error(MG_ERR_INVALID_ARG, "mg_cg_solve_noalloc: null argument");
  if (!(rtol > 0.0) || maxit < 0)
    return set_error(MG_ERR_INVALID_ARG, "mg_cg_solve_noalloc: rtol must be > 0, maxit >= 0");
  if (p->ndof > MG_CG_NOALLOC_MAX_NDOF)
    return set_error(MG_ERR_SIZE, "mg_cg_solve_noalloc: ndof " + std::to_string(p->ndof) +
                                      " exceeds MG_CG_NOALLOC_MAX_NDOF (" +
                                      std::to_string(MG_CG_NOALLOC_MAX_NDOF) + ") of the fixed work array");
  if (!p->on_device)
    return set_error(MG_ERR_INVALID_ARG,
                     "mg_cg_solve_noalloc: the plan is not resident on the device yet (make one regular GPU call "
                     "on it first, e.g. mg_assemble)");
  if (cg_work_bytes<double>(p->ndof) > kNoAllocScratchBytes)
    return set_error(MG_ERR_SIZE, "mg_cg_solve_noalloc: work space above the fixed array");
  // the scratch address below is the current device's; the plan's arrays must be there too
  MG_TRY(check_device(p->mesh->device, "mg_cg_solve_noalloc: the plan"));
  void* base = nullptr;
  MG_TRY(noalloc_scratch(&base));
  cudaStream_t st = (cudaStream_t)stream;
  CgWork<double> w = cg_work_carve<double>(base, p->ndof);
  const int G = CgShape<double>::group(p), nb = CgShape<double>::blocks(p, G);
  const int64_t n = p->ndof;
  const int vb = vec_blocks<double>(n);
  const auto t0 = std::chrono::steady_clock::now();
  // cg_start writes the scalars from the host (tickets and flags start at zero)
  MG_TRY(cg_start<double>(p, d_values, d_b, d_x, 0, precond == MG_PREC_JACOBI, rtol, maxit, w, G, nb, st));
  CgScalars hs{};
  for (int launched = 0;; launched += kGraphIters) {
    for (int k = 0; k < kGraphIters; ++k) {
      constexpr bool pdl = CgShape<double>::pdl;
      if (p->d_coloff) {
        MG_DISPATCH_G(G, (launch_k(pdl, k_cg_spmv<double, g, int16_t>, nb, kSolveThreads, st, n,
                                   (const int32_t*)p->d_rowptr, (const int16_t*)p->d_coloff, d_values,
                                   (const double*)w.p, w.q, w.partials, w.s)));
      } else {
        MG_DISPATCH_G(G, (launch_k(pdl, k_cg_spmv<double, g, int32_t>, nb, kSolveThreads, st, n,
                                   (const int32_t*)p->d_rowptr, (const int32_t*)p->d_colind, d_values,
                                   (const double*)w.p, w.q, w.partials, w.s)));
      }
      launch_k(pdl, k_cg_update<double>, vb, kSolveThreads, st, n, d_x, w.r, w.z, (const double*)w.p,
               (const double*)w.q, (const double*)w.dinv, w.partials, w.s);
      launch_k(pdl, k_cg_dir<double>, vb, kSolveThreads, st, n, (const double*)w.z, w.p, (const CgScalars*)w.s);
    }
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaMemcpyAsync(&hs, w.s, sizeof(CgScalars), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    if (hs.done) break;
    if (launched + kGraphIters > maxit + kGraphIters) break;
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info) {
    info->iterations = hs.iter;
    info->outer_iterations = 0;
    info->converged = hs.done == 1;
    info->rel_residual = rel_residual(hs.rr, hs.bb);
    info->seconds = secs;
  }
  if (hs.done == 2) return set_error(MG_ERR_NOT_CONVERGED, "CG breakdown: p.Ap <= 0");
  if (hs.done != 1) return set_error(MG_ERR_NOT_CONVERGED, "CG reached maxit");
  return MG_OK;
}

mg_status mg_spmv(mg_plan* plan, int32_t prec, const void* d_values, const void* d_x, void* d_y, void* stream)
{
  NvtxRange nvtx_range("mg_spmv");
  if (!plan) return set_error(MG_ERR_INVALID_ARG, "mg_spmv: null plan");
  return launch_spmv(plan, prec, d_values, d_x, d_y, (cudaStream_t)stream);
}

mg_status mg_cg_solve(mg_plan* p, const double* d_values, const double* d_b, double* d_x, double rtol,
                      int32_t maxit, int32_t precond, mg_cg_info* info, void* stream)
{
  NvtxRange nvtx_range("mg_cg_solve");
  if (!p || !d_values || !d_b || !d_x) return set_error(MG_ERR_INVALID_ARG, "mg_cg_solve: null argument");
  if (!(rtol > 0.0) || maxit < 0) return set_error(MG_ERR_INVALID_ARG, "mg_cg_solve: rtol must be > 0, maxit >= 0");
  MG_TRY(plan_device(p));
  cudaStream_t st = (cudaStream_t)stream;
  void* base = nullptr;
  MG_TRY(plan_work(p, cg_work_bytes<double>(p->ndof), &base));
  CgWork<double> w = cg_work_carve<double>(base, p->ndof);
  const int G = CgShape<double>::group(p), nb = CgShape<double>::blocks(p, G);
  cudaEvent_t e0, e1;
  MG_CUDA(cudaEventCreate(&e0));
  MG_CUDA(cudaEventCreate(&e1));
  MG_CUDA(cudaEventRecord(e0, st));
  CgScalars* hs = reinterpret_cast<CgScalars*>(p->h_pinned);
  mg_status s = cg_start<double>(p, d_values, d_b, d_x, 0, precond == MG_PREC_JACOBI, rtol, maxit, w, G, nb, st);
  if (s == MG_OK) s = cg_iterate<double>(p, d_values, d_x, w, G, nb, maxit, st, hs);
  MG_CUDA(cudaEventRecord(e1, st));
  MG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != MG_OK) return s;
  MG_CUDA(cudaMemcpy(hs, w.s, sizeof(CgScalars), cudaMemcpyDeviceToHost));
  if (info) {
    info->iterations = hs->iter;
    info->outer_iterations = 0;
    info->converged = hs->done == 1;
    info->rel_residual = rel_residual(hs->rr, hs->bb);
    info->seconds = ms * 1e-3;
  }
  if (hs->done == 2) return set_error(MG_ERR_NOT_CONVERGED, "CG breakdown: p.Ap <= 0");
  if (hs->done != 1) return set_error(MG_ERR_NOT_CONVERGED, "CG reached maxit");
  return MG_OK;
}

mg_status mg_cg_refined(mg_plan* p, const double* d_values64, const float* d_values32, const double* d_b,
                        double* d_x, double rtol, int32_t max_outer, int32_t max_inner, double inner_rtol,
                        int32_t precond, mg_cg_info* info, void* stream)
{
  NvtxRange nvtx_range("mg_cg_refined");
  if (!p || !d_values64 || !d_values32 || !d_b || !d_x)
    return set_error(MG_ERR_INVALID_ARG, "mg_cg_refined: null argument");
  if (!(rtol > 0.0) || !(inner_rtol > 0.0) || !(inner_rtol < 1.0) || max_outer < 1 || max_inner < 1)
    return set_error(MG_ERR_INVALID_ARG, "mg_cg_refined: bad tolerance or iteration limits");
  MG_TRY(plan_device(p));
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = p->ndof;
  // layout: [CgWork<float>][r64][x32][scalars of the FP64 residual]
  const size_t wbytes = cg_work_bytes<float>(n);
  const size_t v64 = ((size_t)n * 8 + 255) / 256 * 256, v32 = ((size_t)n * 4 + 255) / 256 * 256;
  void* base = nullptr;
  MG_TRY(plan_work(p, wbytes + v64 + v32 + 256, &base));
  CgWork<float> w = cg_work_carve<float>(base, n);
  double* r64 = (double*)((char*)base + wbytes);
  float* x32 = (float*)((char*)r64 + v64);
  CgScalars* s64 = (CgScalars*)((char*)x32 + v32);
  const int G64 = CgShape<double>::group(p), nb64 = CgShape<double>::blocks(p, G64);
  const int G = CgShape<float>::group(p), nb = CgShape<float>::blocks(p, G);
  const int eb = vec_blocks<float>(n);
  CgScalars* hs = reinterpret_cast<CgScalars*>(p->h_pinned);
  cudaEvent_t e0, e1;
  MG_CUDA(cudaEventCreate(&e0));
  MG_CUDA(cudaEventCreate(&e1));
  MG_CUDA(cudaEventRecord(e0, st));
  int anchors = 0, inner = 0;
  bool converged = false;
  double relres = INFINITY, bb64 = 1.0;
  mg_status s = MG_OK;
  // FP64 residual of the current x (into r64, s64->rr, s64->bb)
  auto residual64 = [&]() -> mg_status {
    MG_CUDA(cudaMemsetAsync(s64, 0, sizeof(CgScalars), st));
    MG_DISPATCH_G(G64, (k_residual64<g><<<nb64, kSolveThreads, 0, st>>>(n, p->d_rowptr, p->d_colind, d_values64,
                                                                          d_b, d_x, r64, w.partials, s64)));
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaMemcpyAsync(hs, s64, sizeof(CgScalars), cudaMemcpyDeviceToHost, st));
    MG_CUDA(cudaStreamSynchronize(st));
    bb64 = hs->bb;
    relres = rel_residual(hs->rr, hs->bb);
    return MG_OK;
  };
  s = residual64();
  if (s == MG_OK && relres <= rtol) converged = true;
  if (s == MG_OK && !converged) {
    // first anchor: a plain FP32 CG start on r32 = r64 (x32 = 0), then the
    // target and the reliable-update trigger in its scalars
    k_scale_cast<<<eb, 256, 0, st>>>(n, r64, 1.0, w.r, x32);
    s = cg_start<float>(p, d_values32, w.r, x32, 1, precond == MG_PREC_JACOBI, 1.0, max_inner, w, G, nb, st);
    if (s == MG_OK) {
      MG_CUDA(cudaMemcpyAsync(hs, w.s, sizeof(CgScalars), cudaMemcpyDeviceToHost, st));
      MG_CUDA(cudaStreamSynchronize(st));
      hs->bb = 1.0;
      hs->tol2 = rtol * rtol * bb64;  // recursive-residual target: ||r|| <= rtol ||b||
      hs->rr_anchor = hs->rr;
      // the FP32 recursion drifts from the true residual beyond ~3 decades
      // between anchors (measured: 1e-4 took 33x the iterations on P2 48^3)
      const double delta = std::max(inner_rtol, kMinAnchorRatio);
      hs->delta2 = delta * delta;
      hs->done = 0;
      MG_CUDA(cudaMemcpyAsync(w.s, hs, sizeof(CgScalars), cudaMemcpyHostToDevice, st));
    }
    while (s == MG_OK) {
      s = cg_iterate<float>(p, d_values32, x32, w, G, nb, max_inner, st, hs);
      if (s != MG_OK) break;
      inner = hs->iter;
      const int why = hs->done;
      if (why == 2) { s = set_error(MG_ERR_NOT_CONVERGED, "refined CG breakdown: p.Ap <= 0"); break; }
      // anchor: x += x32, r64 = b - A64 x
      k_anchor_x<<<eb, 256, 0, st>>>(n, d_x, x32);
      ++anchors;
      s = residual64();
      if (s != MG_OK) break;
      if (relres <= rtol) { converged = true; break; }
      if (why == 3 || anchors >= max_outer) break;
      // replace the FP32 residual, keep the direction, resume
      k_anchor_r<<<eb, kSolveThreads, 0, st>>>(n, r64, w.r, w.z, w.dinv, w.partials, w.s);
      launch_k(false, k_cg_dir<float>, eb, kSolveThreads, st, n, (const float*)w.z, w.p, (const CgScalars*)w.s);
      MG_CUDA(cudaGetLastError());
    }
  }
  MG_CUDA(cudaEventRecord(e1, st));
  MG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != MG_OK) return s;
  if (info) {
    info->iterations = inner;
    info->outer_iterations = anchors;
    info->converged = converged;
    info->rel_residual = relres;
    info->seconds = ms * 1e-3;
  }
  if (!converged) return set_error(MG_ERR_NOT_CONVERGED, "refined CG: no convergence within max_outer / max_inner");
  return MG_OK;
}

}  // extern "C"
