// Assembly kernels for sm_103a: element matrices of the P1/P2 bilinear forms
// reduced straight into CSR values, plus the Dirichlet elimination, the
// adjoint-gradient kernel and the load vector.
//
// k_assemble is a persistent kernel: each CTA repeatedly takes the next block of
// rows (an integer work counter) and, for every chunk of the block's elements,
//   stage    a bulk copy (cp.async.bulk, completion on an mbarrier) brings the
//            chunk's element nodes and element ranks into shared memory while the
//            previous chunk is reduced, and the chunk's contribution words while
//            its element matrices are computed;
//   phase 1  one thread per P1 element (eight per P2 element) computes the
//            symmetric element matrix into shared memory, entry-major;
//   phase 2  every thread walks its own slot-sorted segments of contribution
//            words and adds each contribution to its accumulator slot -- within
//            a chunk a slot belongs to exactly one thread.
// The owned rows are then written to their contiguous CSR ranges.  No atomics
// touch values; the per-slot summation order is fixed by the plan, so the
// results are bitwise reproducible.
//
// Element math (reference: src/morganaIntegrator/integratorOEL3d_STD.hpp:106-137,
// src/morganaOperators/opEL3dA.hpp:129-165, opEL3dF.hpp:102-133, opEL3dG.hpp:83-108,
// opEL3dM.hpp:129-158, src/morganaFields/fePr3d.hpp:418-442,643-667 in morganaPublic).
// The tetrahedron map is affine, so J, detJ and J^-1 are the same at every
// quadrature point and the quadrature loop folds into reference tables:
//   stiffness  K_ij = coef det sum_q w_q (J^-T g^_i)(J^-T g^_j)
//                   = (coef / det) sum_{a<=b} (C_a . C_b) T^{ab}_ij ,
//              C_a the columns of the cofactor matrix of J (adj J = C^T),
//              T^{ab} = sum_q w_q g^_ia g^_jb (symmetrised for a != b);
//   P1         the reference gradients are constant, so for i, j >= 1
//              K_ij = coef sum_q w_q / det (C_{i-1} . C_{j-1}), and the row of
//              vertex 0 follows from the zero row sums of a stiffness matrix;
//   mass       K_ij = coef det sum_q w_q phi^_i phi^_j.
// detJ is signed, as in the reference (positive on checked meshes).
//
// Arithmetic modes: kF32 (FP32 values), kDW (FP64-accurate values from
// double-word float arithmetic on the FP32 pipes, written as IEEE doubles), kF64
// (native FP64).  GB300 runs FP64 at ~1/60 of its FP32 rate, so MG_F64 uses kDW;
// MG_F64_NATIVE selects kF64 (the full FP64 exponent range).
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "mg_ff.cuh"
#include "mg_internal.h"

namespace mg {

enum { kF32 = 0, kDW = 1, kF64 = 2 };

// ---------------------------------------------------------- double-word ops --
__device__ __forceinline__ ff operator+(ff a, ff b) { return ff_add_s(a, b); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return ff_add_s(a, ff_neg(b)); }
__device__ __forceinline__ ff operator-(ff a) { return ff_neg(a); }
__device__ __forceinline__ ff operator*(ff a, ff b) { return ff_mul(a, b); }
__device__ __forceinline__ ff operator/(ff a, ff b) { return ff_div(a, b); }

// An element's scale factor inside the range where the double-word assembly is
// FP64-accurate: zero, or |v| in 2^-96 .. 2^112 (the error terms of products
// stay normal floats and no intermediate overflows).
__device__ __forceinline__ bool dw_scale_ok(ff v)
{
  const uint32_t ex = (__float_as_uint(v.hi) >> 23) & 0xffu;
  return v.hi == 0.0f || (ex >= 127u - 96u && ex <= 127u + 112u);
}

template <int MODE> struct Arith;
// sum_into(s, x): s += x for the phase-2 sums.  The double-word form defers
// renormalisation: the high words are added error-free (two_sum), the low
// words and errors collect in s.lo, which may exceed half an ulp of s.hi (the
// final hi + lo is formed in FP64 when the value is written).
template <> struct Arith<kF32> {
  using T = float;
  __device__ static void sum_into(T& s, T x) { s += x; }
  using Out = float;
  // double -> float by integer operations (the conversion instruction runs on
  // the FP64 pipe): hi + lo of the double-word split, rounded once
  __device__ static T from(double x)
  {
    const ff t = ff_from_double_bits(x);
    return __fadd_rn(t.hi, t.lo);
  }
  __device__ static T zero() { return 0.0f; }
  __device__ static Out out(T v) { return v; }
};
template <> struct Arith<kDW> {
  using T = ff;
  __device__ static void sum_into(T& s, T x)
  {
    const ff t = two_sum(s.hi, x.hi);
    s.hi = t.hi;
    s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, x.lo));
  }
  using Out = double;
  __device__ static T from(double x) { return ff_from_double_bits(x); }
  __device__ static T zero() { return ff{0.0f, 0.0f}; }
  __device__ static Out out(T v) { return ff_to_double_int(v); }
};
template <> struct Arith<kF64> {
  using T = double;
  __device__ static void sum_into(T& s, T x) { s += x; }
  using Out = double;
  __device__ static T from(double x) { return x; }
  __device__ static T zero() { return 0.0; }
  __device__ static Out out(T v) { return v; }
};

// ------------------------------------------------------------ PTX helpers --
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same buffers.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16),
// completion signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Bounded wait: gives up after `limit` polls (each poll may suspend the thread
// for a short, hardware-chosen time) and returns false.  The pipeline waits take
// the plan's limit (kWaitLimit unless a diagnostic lowered it); the producer's
// final waits for its own copies in flight always take kWaitLimit, so that no
// bulk copy is still writing shared memory when the CTA exits.
constexpr uint32_t kWaitLimit = MG_WAIT_LIMIT_DEFAULT;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit)
{
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

enum { kDevErrTimeout = 1 };

// ---------------------------------------------------------------- geometry --
template <typename T>
struct Cof {
  T c[3][3];  // cofactor matrix C[r][k] of J; column a of C = det * (J^-T e_a)
  T det;
};

template <typename T>
__device__ __forceinline__ void cofactors(const T J[3][3], Cof<T>& f)
{
  f.c[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  f.c[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  f.c[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  f.c[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  f.c[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  f.c[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  f.c[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  f.c[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  f.c[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  f.det = J[0][0] * f.c[0][0] + J[0][1] * f.c[0][1] + J[0][2] * f.c[0][2];
}

struct GeoPtrs {
  const double4_32a* xyz;  // (x, y, z, 0)
  const float4* rec;       // 2 per node: (hx, hy, hz, mx), (my, mz, lx, ly)
  const float* loz;        // lz
};

// The coordinates an element needs.  The assembly kernel reads them from the
// chunk record staged in shared memory: per distinct vertex of the chunk, its
// coordinates relative to the chunk's first vertex split exactly into three
// floats r = hi + mid + lo, in the layout of the mesh's absolute records
// (a = hi.xyz mid.x, b = mid.yz lo.xy, c = lo.z).  An edge vector r_k - r_0 is
// then the exact difference of the mesh's FP64 coordinates -- the reference's J,
// which geoMapInterface::getGradient forms as x_k - x_0 -- up to the rounding of
// the arithmetic that forms it.  (A two-float split kept 2^-48 of the chunk's
// extent, several edges; a cancelling cofactor amplified that past 1e-12 on
// strongly jittered 128^3 meshes.)  The adjoint kernel reads the mesh's absolute
// records from global memory.
struct StagedVerts {
  const float4* a;  // hi.xyz, mid.x
  const float4* b;  // mid.y, mid.z, lo.x, lo.y
  const float* c;   // lo.z
};
struct FetchAbs {  // four vertices in the three-float form (staged or absolute)
  float4 a[4], b[4];
  float lz[4];
};
template <int MODE> struct Fetch;
template <> struct Fetch<kF64> {
  double4_32a x[4];
};

__device__ __forceinline__ void fetch(const GeoPtrs& g, int4 n, FetchAbs& F)
{
  const int id[4] = {n.x, n.y, n.z, n.w};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    F.a[s] = g.rec[2 * (int64_t)id[s]];
    F.b[s] = g.rec[2 * (int64_t)id[s] + 1];
    F.lz[s] = g.loz[id[s]];
  }
}

// the four vertices of an item from a staged record (LO: the third floats too;
// the FP32 arithmetic needs hi + mid only)
template <bool LO>
__device__ __forceinline__ void fetch_staged(const StagedVerts& v, ushort4 lc, FetchAbs& F)
{
  const int id[4] = {lc.x, lc.y, lc.z, lc.w};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    F.a[s] = v.a[id[s]];
    F.b[s] = v.b[id[s]];
    F.lz[s] = LO ? v.c[id[s]] : 0.0f;
  }
}

// components of a three-float record: hi, mid, lo
__device__ __forceinline__ float rec_hi(const float4& a, int r) { return r == 0 ? a.x : (r == 1 ? a.y : a.z); }
__device__ __forceinline__ float rec_mid(const float4& a, const float4& b, int r) { return r == 0 ? a.w : (r == 1 ? b.x : b.y); }
__device__ __forceinline__ float rec_lo(const float4& b, float lz, int r) { return r == 0 ? b.z : (r == 1 ? b.w : lz); }
// the coordinate as a double: hi + mid + lo, every partial sum exact
__device__ __forceinline__ double rec_x(const float4& a, const float4& b, float lz, int r)
{
  return ((double)rec_hi(a, r) + (double)rec_mid(a, b, r)) + (double)rec_lo(b, lz, r);
}

__device__ __forceinline__ double comp(const double4_32a& v, int r) { return r == 0 ? v.x : (r == 1 ? v.y : v.z); }

__device__ __forceinline__ void geometry(const Fetch<kF64>& F, Cof<double>& f)
{
  double J[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) J[r][k] = comp(F.x[k + 1], r) - comp(F.x[0], r);
  cofactors<double>(J, f);
}

// Near-degenerate elements.  The determinant is a cofactor expansion; when its
// terms cancel (sum_k |J0k C0k| > kCancelTol |det|) the relative error of det,
// and of every entry scaled by 1/det, is that many times the arithmetic's own
// (measured on GB300: double-word 2.3e-12 and FP32 7e-6 against the FP64 oracle
// at a cancellation of ~230).  Such elements recompute J, the cofactors and det
// in FP64 from the staged coordinates -- out of line, so that the rare FP64
// path does not occupy the FP64 pipe of every other element.
constexpr float kCancelTol = 16.0f;

template <typename T>
__device__ __forceinline__ float hi_of(const T& v);
template <>
__device__ __forceinline__ float hi_of<float>(const float& v) { return v; }
template <>
__device__ __forceinline__ float hi_of<ff>(const ff& v) { return v.hi; }

template <>
__device__ __forceinline__ float hi_of<double>(const double& v) { return (float)v; }

// P1 stiffness needs the gradient of every vertex: the columns C_0..C_3 of the
// cofactor matrix (gradients times det).  C_1..C_3 come from the edge vectors at
// vertex 0.  C_0:
//  - FP32: formed for every element from the face opposite vertex 0,
//    (x3 - x1) x (x2 - x1), accurate to its own magnitude -- cheap in FP32, and
//    the zero-row-sum form C_0 = -(C_1 + C_2 + C_3) would cost eps |C_max| / |C_0|
//    relative on the entries of vertex 0, too much at FP32's eps;
//  - double-word: the zero-row-sum form (eps 2^-47).
// Elements whose gradients differ by more than 8x (|C_max| > 8 |C_min| over all
// four, or a cancelling determinant) take the rare path staged_rare_stiffness: a
// cofactor is a 2x2 minor whose terms then cancel by about that ratio, and so does
// the zero-row sum; the rare path computes the geometry in FP64 from the exact
// coordinates, as the reference does.  On a Kuhn cube jittered by 0.25 h (12.6 M
// tets, ratios up to 21) ~0.01 % of the elements are rare.
enum { kP1Common = 0, kP1Fp64 = 1 };

template <typename T>
__device__ __forceinline__ int p1_class(const Cof<T>& f)
{
  float n[4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float na = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) na = fmaf(hi_of(f.c[r][a]), hi_of(f.c[r][a]), na);
    n[a + 1] = na;
  }
  n[0] = 0.0f;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const float s = hi_of(f.c[r][0]) + hi_of(f.c[r][1]) + hi_of(f.c[r][2]);
    n[0] = fmaf(s, s, n[0]);
  }
  const float nmax = fmaxf(fmaxf(n[0], n[1]), fmaxf(n[2], n[3]));
  const float nmin = fminf(fminf(n[0], n[1]), fminf(n[2], n[3]));
  return nmax > 64.0f * nmin ? kP1Fp64 : kP1Common;
}

// |det| small against its expansion terms
template <typename T>
__device__ __forceinline__ bool det_cancels(const T J[3][3], const Cof<T>& f)
{
  const float t = fabsf(hi_of(J[0][0]) * hi_of(f.c[0][0])) + fabsf(hi_of(J[0][1]) * hi_of(f.c[0][1])) +
                  fabsf(hi_of(J[0][2]) * hi_of(f.c[0][2]));
  return t > kCancelTol * fabsf(hi_of(f.det));
}

__device__ __forceinline__ void store_geometry(const Cof<double>& d, Cof<float>& f)
{
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) f.c[r][k] = (float)d.c[r][k];
  f.det = (float)d.det;
}
__device__ __forceinline__ void store_geometry(const Cof<double>& d, Cof<ff>& f)
{
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) f.c[r][k] = ff_from_double_bits(d.c[r][k]);
  f.det = ff_from_double_bits(d.det);
}
__device__ __forceinline__ void store_geometry(const Cof<double>& d, Cof<double>& f) { f = d; }

template <typename T> __device__ __forceinline__ T from_double(double x);
template <> __device__ __forceinline__ float from_double<float>(double x) { return (float)x; }
template <> __device__ __forceinline__ ff from_double<ff>(double x) { return ff_from_double_bits(x); }
template <> __device__ __forceinline__ double from_double<double>(double x) { return x; }

// Double-word cofactors and determinant from double-word edge vectors.
__device__ __forceinline__ void dw_cofactors(const ff J[3][3], Cof<ff>& f)
{
  f.c[0][0] = ff_cross(J[1][1], J[2][2], J[1][2], J[2][1]);
  f.c[0][1] = ff_cross(J[1][2], J[2][0], J[1][0], J[2][2]);
  f.c[0][2] = ff_cross(J[1][0], J[2][1], J[1][1], J[2][0]);
  f.c[1][0] = ff_cross(J[0][2], J[2][1], J[0][1], J[2][2]);
  f.c[1][1] = ff_cross(J[0][0], J[2][2], J[0][2], J[2][0]);
  f.c[1][2] = ff_cross(J[0][1], J[2][0], J[0][0], J[2][1]);
  f.c[2][0] = ff_cross(J[0][1], J[1][2], J[0][2], J[1][1]);
  f.c[2][1] = ff_cross(J[0][2], J[1][0], J[0][0], J[1][2]);
  f.c[2][2] = ff_cross(J[0][0], J[1][1], J[0][1], J[1][0]);
  f.det = ff_dot3(J[0], f.c[0]);
}

// Double-word difference of two three-float numbers x = hi + mid + lo:
// x_b - x_a = (hi_b - hi_a) + (mid_b - mid_a) + (lo_b - lo_a) with the two
// leading differences error-free -- relative error ~2^-47 of the difference.
__device__ __forceinline__ ff dw_diff3(float hb, float ha, float mb, float ma, float lb, float la)
{
  const ff s1 = two_sum(hb, -ha);
  const ff s2 = two_sum(mb, -ma);
  const ff s = two_sum(s1.hi, s2.hi);
  const float t = __fadd_rn(__fadd_rn(__fadd_rn(s.lo, s1.lo), s2.lo), __fsub_rn(lb, la));
  return two_sum(s.hi, t);
}
// component r of the edge from vertex j to vertex k, double-word and FP32, from
// hi + mid only (48 bits of the chunk-relative coordinate): the common path,
// whose elements (gradient ratios <= 8, p1_class) do not amplify that
// truncation past ~1e-13
__device__ __forceinline__ ff dw_edge2(const FetchAbs& F, int k, int j, int r)
{
  const ff s1 = two_sum(rec_hi(F.a[k], r), -rec_hi(F.a[j], r));
  return two_sum(s1.hi, __fadd_rn(s1.lo, __fsub_rn(rec_mid(F.a[k], F.b[k], r), rec_mid(F.a[j], F.b[j], r))));
}
__device__ __forceinline__ float f32_edge(const FetchAbs& F, int k, int j, int r)
{
  return (rec_hi(F.a[k], r) - rec_hi(F.a[j], r)) + (rec_mid(F.a[k], F.b[k], r) - rec_mid(F.a[j], F.b[j], r));
}

// FP64 geometry from three-float coordinates (exact as doubles)
__device__ __forceinline__ void geometry_fp64(const FetchAbs& F, Cof<double>& d)
{
  Fetch<kF64> D;
#pragma unroll
  for (int s = 0; s < 4; ++s)
    D.x[s] = make_double4_32a(rec_x(F.a[s], F.b[s], F.lz[s], 0), rec_x(F.a[s], F.b[s], F.lz[s], 1),
                              rec_x(F.a[s], F.b[s], F.lz[s], 2), 0.0);
  geometry(D, d);
}

// The common path: geometry of a staged item in the mode's arithmetic, reading
// vertex 0 and then one vertex per edge column (fewer live registers than all
// four at once); returns whether the element needs the FP64 geometry
// (det_cancels).  FP32: edge vectors (hi_k - hi_0) + (mid_k - mid_0), to a float
// ulp of the edge; double-word: dw_edge2 of hi + mid.  With c0 (FP32 P1
// stiffness) also C_0 = (x3 - x1) x (x2 - x1) from the edge columns,
// x_k - x_1 = J_k - J_1: on the common path (gradient ratios <= 8, p1_class) the
// face edges are within a few float ulps, and no vertex is read twice.
template <int MODE>
__device__ __forceinline__ bool geometry_staged_lazy(const StagedVerts& v, ushort4 lc, Cof<typename Arith<MODE>::T>& f,
                                                     float* c0 = nullptr)
{
  using T = typename Arith<MODE>::T;
  constexpr bool LO = MODE == kF64;
  FetchAbs F;  // slots 0 (vertex 0) and 1 (the current column's vertex) only
  F.a[0] = v.a[lc.x];
  F.b[0] = v.b[lc.x];
  F.lz[0] = LO ? v.c[lc.x] : 0.0f;
  T J[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int id = k == 0 ? lc.y : (k == 1 ? lc.z : lc.w);
    F.a[1] = v.a[id];
    F.b[1] = v.b[id];
    F.lz[1] = LO ? v.c[id] : 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      if constexpr (MODE == kF32) J[r][k] = f32_edge(F, 1, 0, r);
      else if constexpr (MODE == kDW) J[r][k] = dw_edge2(F, 1, 0, r);
      else J[r][k] = rec_x(F.a[1], F.b[1], F.lz[1], r) - rec_x(F.a[0], F.b[0], F.lz[0], r);
    }
  }
  if constexpr (MODE == kDW) dw_cofactors(J, f);
  else cofactors<T>(J, f);
  if constexpr (MODE == kF32) {
    if (c0) {
      float f2[3], f3[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        f2[r] = J[r][1] - J[r][0];
        f3[r] = J[r][2] - J[r][0];
      }
      c0[0] = f3[1] * f2[2] - f3[2] * f2[1];
      c0[1] = f3[2] * f2[0] - f3[0] * f2[2];
      c0[2] = f3[0] * f2[1] - f3[1] * f2[0];
    }
  }
  if constexpr (MODE == kF64) return false;
  else return det_cancels<T>(J, f);
}

// Near-degenerate elements: the FP64 geometry of a staged item, out of line and
// returned by value (no register of the caller is passed by address).
template <typename T>
static __device__ __noinline__ Cof<T> staged_geometry_fp64(StagedVerts v, ushort4 lc)
{
  FetchAbs D;
  fetch_staged<true>(v, lc, D);
  Cof<double> g;
  geometry_fp64(D, g);
  Cof<T> f;
  store_geometry(g, f);
  return f;
}

// near-degenerate elements: FP64 geometry from the mesh's FP64 coordinates
static __device__ __noinline__ void recompute_fp64_abs(const GeoPtrs& g, int4 n, Cof<ff>& f)
{
  Fetch<kF64> D;
  const int id[4] = {n.x, n.y, n.z, n.w};
  for (int s = 0; s < 4; ++s) D.x[s] = g.xyz[id[s]];
  Cof<double> d;
  geometry(D, d);
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) f.c[r][k] = ff_from_double_bits(d.c[r][k]);
  f.det = ff_from_double_bits(d.det);
}

__device__ __forceinline__ void geometry_abs(const GeoPtrs& g, int4 n, Cof<ff>& f)
{
  FetchAbs F;
  fetch(g, n, F);
  ff J[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      J[r][k] = dw_diff3(rec_hi(F.a[k + 1], r), rec_hi(F.a[0], r), rec_mid(F.a[k + 1], F.b[k + 1], r),
                         rec_mid(F.a[0], F.b[0], r), rec_lo(F.b[k + 1], F.lz[k + 1], r), rec_lo(F.b[0], F.lz[0], r));
  dw_cofactors(J, f);
  if (det_cancels<ff>(J, f)) recompute_fp64_abs(g, n, f);
}

// ------------------------------------------------------- element matrices --
// P1 stiffness, unique entries in sym_index order:
// (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)
template <typename T>
__device__ __forceinline__ void p1_stiff_unique(const Cof<T>& f, T s, T K[10])
{
  T d[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      d[a][b] = s * (f.c[0][a] * f.c[0][b] + f.c[1][a] * f.c[1][b] + f.c[2][a] * f.c[2][b]);
      d[b][a] = d[a][b];
    }
  K[4] = d[0][0];
  K[5] = d[0][1];
  K[6] = d[0][2];
  K[7] = d[1][1];
  K[8] = d[1][2];
  K[9] = d[2][2];
  K[1] = -(d[0][0] + d[1][0] + d[2][0]);  // rows sum to zero
  K[2] = -(d[0][1] + d[1][1] + d[2][1]);
  K[3] = -(d[0][2] + d[1][2] + d[2][2]);
  K[0] = -(K[1] + K[2] + K[3]);
}

template <>
__device__ __forceinline__ void p1_stiff_unique<ff>(const Cof<ff>& f, ff s, ff K[10])
{
  ff col[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r) col[a][r] = f.c[r][a];
  ff d[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      d[a][b] = ff_mul(s, ff_dot3(col[a], col[b]));
      d[b][a] = d[a][b];
    }
  K[4] = d[0][0];
  K[5] = d[0][1];
  K[6] = d[0][2];
  K[7] = d[1][1];
  K[8] = d[1][2];
  K[9] = d[2][2];
  K[1] = -(d[0][0] + d[1][0] + d[2][0]);
  K[2] = -(d[0][1] + d[1][1] + d[2][1]);
  K[3] = -(d[0][2] + d[1][2] + d[2][2]);
  K[0] = -(K[1] + K[2] + K[3]);
}

// C_0 = (x3 - x1) x (x2 - x1) (= -(C_1 + C_2 + C_3)) in FP64 from the exact
// staged coordinates (the rare path): the edges of the face opposite vertex 0,
// then their cross product, accurate to its own magnitude.
__device__ __forceinline__ void staged_c0(const FetchAbs& F, double C0[3])
{
  double f2[3], f3[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const double x1 = rec_x(F.a[1], F.b[1], F.lz[1], r);
    f2[r] = rec_x(F.a[2], F.b[2], F.lz[2], r) - x1;
    f3[r] = rec_x(F.a[3], F.b[3], F.lz[3], r) - x1;
  }
  C0[0] = f3[1] * f2[2] - f3[2] * f2[1];
  C0[1] = f3[2] * f2[0] - f3[0] * f2[2];
  C0[2] = f3[0] * f2[1] - f3[1] * f2[0];
}

// P1 stiffness with every vertex gradient explicit: C_0 given, the entries of
// vertex 0 as s (C_0 . C_j); the others as in p1_stiff_unique.
template <typename T>
__device__ __forceinline__ void p1_stiff_direct(const Cof<T>& f, const T C0[3], T s, T K[10])
{
  T d[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      d[a][b] = s * (f.c[0][a] * f.c[0][b] + f.c[1][a] * f.c[1][b] + f.c[2][a] * f.c[2][b]);
      d[b][a] = d[a][b];
    }
  K[0] = s * (C0[0] * C0[0] + C0[1] * C0[1] + C0[2] * C0[2]);
#pragma unroll
  for (int b = 0; b < 3; ++b) K[1 + b] = s * (C0[0] * f.c[0][b] + C0[1] * f.c[1][b] + C0[2] * f.c[2][b]);
  K[4] = d[0][0];
  K[5] = d[0][1];
  K[6] = d[0][2];
  K[7] = d[1][1];
  K[8] = d[1][2];
  K[9] = d[2][2];
}
template <>
__device__ __forceinline__ void p1_stiff_direct<ff>(const Cof<ff>& f, const ff C0[3], ff s, ff K[10])
{
  ff col[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r) col[a][r] = f.c[r][a];
  K[0] = ff_mul(s, ff_dot3(C0, C0));
#pragma unroll
  for (int b = 0; b < 3; ++b) K[1 + b] = ff_mul(s, ff_dot3(C0, col[b]));
  K[4] = ff_mul(s, ff_dot3(col[0], col[0]));
  K[5] = ff_mul(s, ff_dot3(col[0], col[1]));
  K[6] = ff_mul(s, ff_dot3(col[0], col[2]));
  K[7] = ff_mul(s, ff_dot3(col[1], col[1]));
  K[8] = ff_mul(s, ff_dot3(col[1], col[2]));
  K[9] = ff_mul(s, ff_dot3(col[2], col[2]));
}

// The rare P1 stiffness elements (p1_class): their geometry in FP64 from the exact
// staged coordinates, C_0 from its own face, returned by value (out of line, and
// no register of the caller is passed by address, so the common path keeps its
// registers).
template <typename T>
struct RareK {
  T K[10];
};
template <int MODE>
static __device__ __noinline__ RareK<typename Arith<MODE>::T> staged_rare_stiffness(StagedVerts v, ushort4 lc,
                                                                                   double coef, double wsum,
                                                                                   uint32_t* flags)
{
  using T = typename Arith<MODE>::T;
  FetchAbs F;
  fetch_staged<true>(v, lc, F);
  Cof<double> d;
  geometry_fp64(F, d);
  double c0[3];
  staged_c0(F, c0);
  Cof<T> f;
  store_geometry(d, f);
  T C0[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) C0[k] = from_double<T>(c0[k]);
  const T s = Arith<MODE>::from(coef) * Arith<MODE>::from(wsum) / f.det;
  RareK<T> r;
  p1_stiff_direct<T>(f, C0, s, r.K);
  if constexpr (MODE == kDW)
    if (!dw_scale_ok(s) || !dw_scale_ok(r.K[4])) atomicOr(flags, 2u);
  return r;
}

// The six scaled metric coefficients s (C_a . C_b), ab = 00,11,22,01,02,12.
template <typename T>
__device__ __forceinline__ void metric(const Cof<T>& f, T s, T g[6])
{
  const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int p = 0; p < 6; ++p)
    g[p] = s * (f.c[0][pa[p]] * f.c[0][pb[p]] + f.c[1][pa[p]] * f.c[1][pb[p]] + f.c[2][pa[p]] * f.c[2][pb[p]]);
}

// sum_{p<6} g[p] tab[p * NU + u] (the P2 metric contraction).  Double-word:
// error-free products of the high words chained with two_sum, the low-order
// terms in one float, one renormalisation (instead of one per operation).
template <typename T>
__device__ __forceinline__ T metric_dot(const T g[6], const T* tab, int NU, int u)
{
  T v = g[0] * tab[u];
#pragma unroll
  for (int k = 1; k < 6; ++k) v = v + g[k] * tab[k * NU + u];
  return v;
}
template <>
__device__ __forceinline__ ff metric_dot<ff>(const ff g[6], const ff* tab, int NU, int u)
{
  const ff t0 = tab[u];
  const ff p0 = two_prod(g[0].hi, t0.hi);
  float hi = p0.hi;
  float lo = __fmaf_rn(g[0].hi, t0.lo, __fmaf_rn(g[0].lo, t0.hi, p0.lo));
#pragma unroll
  for (int k = 1; k < 6; ++k) {
    const ff t = tab[k * NU + u];
    const ff q = two_prod(g[k].hi, t.hi);
    const ff s = two_sum(hi, q.hi);
    hi = s.hi;
    lo = __fadd_rn(lo, __fadd_rn(s.lo, __fmaf_rn(g[k].hi, t.lo, __fmaf_rn(g[k].lo, t.hi, q.lo))));
  }
  return two_sum(hi, lo);
}

struct AsmArgs {
  const BlockDesc* blocks;
  const unsigned char* chunk_data;  // chunk records (layout at ChunkDesc)
  const int2* chunk_rec;            // (offset / 16, bytes) per chunk
  const int64_t* chunk_wb;          // first contribution word of each chunk (n_chunks + 1; contiguous)
  const uint32_t* entries;
  const int2* row_meta;             // (accumulator base, CSR start - base) per owned row
  const double* coeff;   // per element in Morton order (indexed by the records' ranks), or null
  double cconst;         // used when coeff is null
  const double* tables;  // unique-entry tables: stiff[6][nu] then mass[nu]
  double wsum;
  void* values;
  uint32_t* counters;
  int nblocks;
  int stiff;
  int ent_cap;           // words of one shared-memory contribution buffer
  int stage_cap;         // bytes of one chunk-record stage (the largest record)
  uint32_t wait_limit;   // polls of a pipeline wait before it gives up (mbar_wait)
};

constexpr size_t align16(size_t n) { return (n + 15) / 16 * 16; }

// Barriers of k_assemble (mbarriers in shared memory).  "full" barriers complete
// when a bulk copy has landed (producer arrival + transaction bytes); "empty"
// barriers when the consumers have finished with a buffer; the token barriers
// hand the right to update the accumulators from one consumer group to the
// next.
enum {
  kBarRecFull = 0,                        // [kRecStages] chunk-record stages
  kBarRecEmpty = kBarRecFull + kRecStages,  // [kRecStages]
  kBarEntFull = kBarRecEmpty + kRecStages,  // [kWordStages] contribution-word stages
  kBarEntEmpty = kBarEntFull + kWordStages,  // [kWordStages]
  kBarMetaFull = kBarEntEmpty + kWordStages, // row metadata of a block
  kBarMetaEmpty = kBarMetaFull + 1,
  kBarBlkFull = kBarMetaEmpty + 1,          // [2] block descriptors
  kBarBlkEmpty = kBarBlkFull + 2,           // [2]
  kBarToken = kBarBlkEmpty + 2,             // [kMaxGroups] group g may run phase 2
  kMaxGroups = 3,
  kNumBars = kBarToken + kMaxGroups
};

// Consumer groups of kThreads threads per CTA, plus one producer warp.  Two
// groups (17 warps: at most 5 on one SM sub-partition, 5 x 32 x 96 of its 16 K
// registers) in every mode.  The kernel takes up to kMaxGroups; three FP32
// groups (25 warps, which caps a thread at 72 registers) were measured slower
// on GB300 at P1 128^3 (0.906 against 0.859 ms; the P1 FP32 element math
// spills at 72 registers) and at P2 48^3 (0.496 against 0.484 ms).
template <int MODE> struct AsmShape {
  static constexpr int groups = 2;
  static constexpr int consumers = groups * kThreads;
  static constexpr int threads = consumers + 32;
  static constexpr int max_regs = 96;
};
static_assert(AsmShape<kF32>::groups <= kMaxGroups && AsmShape<kDW>::groups <= kMaxGroups, "token barriers");

// Shared-memory layout of k_assemble.  Every region starts on a 16-byte
// boundary: the bulk copies (chunk records, contribution words, row metadata)
// require 16-byte aligned destinations, the mbarriers 8-byte.
template <int ORDER, int MODE>
struct AsmLayout {
  using T = typename Arith<MODE>::T;
  static constexpr int NB = ORDER == 1 ? 4 : 10;
  static constexpr int NU = ORDER == 1 ? 10 : 55;
  static constexpr int CI = ORDER == 1 ? kChunkP1 : kChunkP2;
  static constexpr size_t acc_bytes = align16(sizeof(T) * (kAccMax + 1));  // + the padding words' dummy slot
  static constexpr size_t buf_bytes = align16(sizeof(T) * (NU * CI + 1));  // per group, + the zero source
  static constexpr size_t tab_bytes = align16(sizeof(T) * 7 * NU);
  // an aligned copy of a block's rows (and the row after) spans at most kRowsMax + 3 entries
  static constexpr size_t meta_bytes = align16(8 * (kRowsMax + 4));
  static constexpr size_t blk_bytes = 2 * sizeof(BlockDesc);
  static constexpr size_t off_buf = acc_bytes;
  static constexpr int G = AsmShape<MODE>::groups;
  static constexpr size_t off_tab = off_buf + G * buf_bytes;
  // P2: per group, the 6 scale factors of each item of a chunk (computed once per item)
  static constexpr size_t geo_bytes = ORDER == 2 ? align16(sizeof(T) * CI * 6) : 0;
  static constexpr size_t off_geo = off_tab + tab_bytes;
  static constexpr size_t off_meta = off_geo + G * geo_bytes;
  static constexpr size_t off_blk = off_meta + meta_bytes;
  static constexpr size_t off_bars = off_blk + blk_bytes;
  static constexpr size_t off_stage = off_bars + align16(8 * kNumBars);
  static_assert(off_buf % 16 == 0 && off_tab % 16 == 0 && off_geo % 16 == 0 && off_meta % 16 == 0 && off_blk % 16 == 0 &&
                    off_bars % 16 == 0 && off_stage % 16 == 0 && buf_bytes % 16 == 0,
                "shared-memory regions must start on 16-byte boundaries");
  __host__ __device__ static size_t stage_bytes(int stage_cap) { return ((size_t)stage_cap + 15) / 16 * 16; }
  __host__ __device__ static size_t words_bytes(int ent_cap) { return ((size_t)ent_cap * 4 + 15) / 16 * 16; }
  __host__ __device__ static size_t off_words(int stage_cap) { return off_stage + kRecStages * stage_bytes(stage_cap); }
  __host__ __device__ static size_t total(int ent_cap, int stage_cap)
  {
    return off_words(stage_cap) + kWordStages * words_bytes(ent_cap);
  }
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Named barriers among consumer threads (the producer warp never takes part):
// id 1 = all consumers, id 2 + g = consumer group g.  The _or forms return the
// OR of `pred` over the participants.
template <int ID, int COUNT>
__device__ __forceinline__ void named_sync()
{
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(COUNT) : "memory");
}
template <int ID, int COUNT>
__device__ __forceinline__ bool named_sync_or(bool pred)
{
  uint32_t r;
  asm volatile(
      "{\n"
      " .reg .pred p, q;\n"
      " setp.ne.u32 p, %1, 0;\n"
      " bar.red.or.pred q, %2, %3, p;\n"
      " selp.u32 %0, 1, 0, q;\n"
      "}\n"
      : "=r"(r)
      : "r"((uint32_t)pred), "n"(ID), "n"(COUNT)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ bool group_sync_or(int g, bool pred)
{
  if (g == 0) return named_sync_or<2, kThreads>(pred);
  if (g == 1) return named_sync_or<3, kThreads>(pred);
  return named_sync_or<4, kThreads>(pred);
}

// k_assemble: a persistent, warp-specialised kernel; per CTA one producer warp
// and G consumer groups of kThreads threads (AsmShape).
//
// The producer (one thread) takes blocks from the work counter and streams, for
// chunk q of the CTA (counted across its blocks), the chunk record into stage
// q % kRecStages and the contribution words into buffer q % 2, then each
// block's row metadata; it waits on an "empty" barrier before reusing a buffer
// and runs several chunks (and across block boundaries) ahead.
//
// Consumer group g takes the chunks q with q % G == g:
//   phase 1    wait record q; gather the element coefficients; element
//              matrices from the staged vertices -> the group's buf
//   barrier    (group) release record q
//   phase 2    wait words q and the token (the previous group finished phase 2
//              of chunk q - 1); add the contributions to the owned slots; pass
//              the token on to the next group
//   barrier    (group) release words q
// so the groups' phase 1 runs beside another group's phase 2, while the
// accumulator updates stay in chunk order (the sums are bitwise reproducible).
// Per block both groups zero the accumulators first and write the owned rows
// last.  Every wait is bounded; after a wait gives up the consumers keep their
// barrier sequence but skip the work, leave together at the end of the block,
// the producer stops issuing and lets its copies in flight land, and the CTA
// records the failure.
template <int ORDER, int MODE>
__global__ void __launch_bounds__(AsmShape<MODE>::threads, 1) __maxnreg__(AsmShape<MODE>::max_regs)
    k_assemble(AsmArgs a)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  using L = AsmLayout<ORDER, MODE>;
  constexpr int kGroups = AsmShape<MODE>::groups, kConsumers = AsmShape<MODE>::consumers;
  constexpr int NU = L::NU, CI = L::CI, NS = kRecStages;
  constexpr int TPI = ORDER == 1 ? 1 : kP2ThreadsPerItem;  // threads per item
  extern __shared__ __align__(16) unsigned char smem[];
  T* acc = reinterpret_cast<T*>(smem);
  T* tab = reinterpret_cast<T*>(smem + L::off_tab);
  int2* smeta = reinterpret_cast<int2*>(smem + L::off_meta);
  BlockDesc* sblk = reinterpret_cast<BlockDesc*>(smem + L::off_blk);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::off_bars);
  unsigned char* stage = smem + L::off_stage;  // [NS][sbytes]
  const int sbytes = (int)L::stage_bytes(a.stage_cap);
  uint32_t* sent = reinterpret_cast<uint32_t*>(smem + L::off_words(a.stage_cap));  // [kWordStages][went]
  const int went = (int)(L::words_bytes(a.ent_cap) / 4);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 7 * NU; i += blockDim.x) tab[i] = A::from(a.tables[i]);
  if (tid == 0) {
    for (int g = 0; g < kGroups; ++g) {
      reinterpret_cast<T*>(smem + L::off_buf + g * L::buf_bytes)[NU * CI] = A::zero();
    }
    for (int k = 0; k < kNumBars; ++k) {
      uint32_t count = 1;
      if (k == kBarBlkEmpty || k == kBarBlkEmpty + 1) count = kConsumers;
      if (k >= kBarToken && k < kBarToken + kMaxGroups) count = kThreads;
      mbar_init(&bars[k], count);
    }
    mbar_fence_init();
  }
  __syncthreads();
  auto stage_of = [&](int q) { return stage + (q % NS) * sbytes; };
  auto desc_of = [&](int q) { return reinterpret_cast<const ChunkDesc*>(stage_of(q)); };
  bool failed = false;

  if (warp == kConsumers / 32) {
    // ------------------------------------------------------------ producer
    // Two lanes with independent waits: lane 0 takes the blocks and streams the
    // contribution words and row metadata, lane 1 the chunk records.  Each runs
    // up to NS (NW) chunks ahead of the consumers, across block boundaries, and
    // waits only on the barrier of its own next copy; the word ranges and record
    // places come from global tables, loaded ahead of those waits.
    if (lane < 2) {
      constexpr int NW = kWordStages;
      int last_rec[NS], last_ent[NW], last_meta = -1;
      for (int s = 0; s < NS; ++s) last_rec[s] = -1;
      for (int s = 0; s < NW; ++s) last_ent[s] = -1;
      auto wait = [&](int k, int parity) {
        if (!failed && !mbar_wait(&bars[k], (uint32_t)parity, a.wait_limit)) failed = true;
        return !failed;
      };
      int q = 0;
      for (int j = 0;; ++j) {
        int b = 0;
        if (lane == 0) b = (int)atomicAdd(&a.counters[0], 1u);
        b = __shfl_sync(0x3u, b, 0);
        BlockDesc d;
        if (b < a.nblocks) {
          d = a.blocks[b];
        } else {
          d = BlockDesc{};
          d.nchunks = -1;  // no more blocks
        }
        if (lane == 0) {
          if (j >= 2 && !wait(kBarBlkEmpty + (j & 1), ((j >> 1) - 1) & 1)) d.nchunks = -1;
          if (!failed) {
            sblk[j & 1] = d;
            mbar_arrive(&bars[kBarBlkFull + (j & 1)]);
          }
        }
        if (__any_sync(0x3u, failed) || d.nchunks < 0) {
          failed = __any_sync(0x3u, failed);
          break;
        }
        const int n = d.nchunks;
        if (lane == 1) {
          // records: chunk c into stage (q + c) % NS once chunk q + c - NS is released
          for (int c = 0; c < n; ++c) {
            const int qq = q + c;
            const int2 r = a.chunk_rec[d.chunk_begin + c];  // lands during the wait
            if (qq >= NS && !wait(kBarRecEmpty + qq % NS, (qq / NS - 1) & 1)) break;
            fence_proxy_async();
            mbar_expect_tx(&bars[kBarRecFull + qq % NS], (uint32_t)r.y);
            bulk_g2s(stage_of(qq), a.chunk_data + (int64_t)r.x * 16, (uint32_t)r.y, &bars[kBarRecFull + qq % NS]);
            last_rec[qq % NS] = qq;
          }
        } else {
          // words: chunk c into stage (q + c) % NW once chunk q + c - NW is released
          for (int c = 0; c < n; ++c) {
            const int qq = q + c;
            const int64_t w0 = a.chunk_wb[d.chunk_begin + c], w1 = a.chunk_wb[d.chunk_begin + c + 1];
            if (qq >= NW && !wait(kBarEntEmpty + qq % NW, (qq / NW - 1) & 1)) break;
            const uint32_t bytes = (uint32_t)(w1 - w0) * 4u;
            fence_proxy_async();
            mbar_expect_tx(&bars[kBarEntFull + qq % NW], bytes);
            if (bytes) bulk_g2s(sent + (qq % NW) * went, a.entries + w0, bytes, &bars[kBarEntFull + qq % NW]);
            last_ent[qq % NW] = qq;
          }
          // the block's row metadata: rows row_begin .. row_begin + row_count and
          // the row after, 16-byte aligned
          if (!failed && (j == 0 || wait(kBarMetaEmpty, (j - 1) & 1))) {
            const int i0 = d.row_begin & ~1, i1 = (d.row_begin + d.row_count + 2) & ~1;
            fence_proxy_async();
            mbar_expect_tx(&bars[kBarMetaFull], (uint32_t)(i1 - i0) * 8u);
            bulk_g2s(smeta, a.row_meta + i0, (uint32_t)(i1 - i0) * 8u, &bars[kBarMetaFull]);
            last_meta = j;
          }
        }
        failed = __any_sync(0x3u, failed);
        if (failed) break;
        q += n;
      }
      if (failed) {
        // let this lane's copies in flight land before the CTA's shared memory goes away
        for (int s = 0; s < NS; ++s)
          if (last_rec[s] >= 0) mbar_wait(&bars[kBarRecFull + s], (uint32_t)((last_rec[s] / NS) & 1), kWaitLimit);
        for (int s = 0; s < NW; ++s)
          if (last_ent[s] >= 0) mbar_wait(&bars[kBarEntFull + s], (uint32_t)((last_ent[s] / NW) & 1), kWaitLimit);
        if (last_meta >= 0) mbar_wait(&bars[kBarMetaFull], (uint32_t)(last_meta & 1), kWaitLimit);
      }
    }
    __syncwarp();
  } else {
    // ----------------------------------------------------------- consumers
    const int g = tid / kThreads;           // group
    const int gtid = tid - g * kThreads;    // thread within the group
    const int gwarp = gtid >> 5;
    // item of the chunk and share of its entries: for P2 the lanes of a warp take
    // the 32 items and the warps the entries (u = warp + 8k), so the entry-major
    // stores buf[u * CI + item] of a warp hit consecutive words (the other way
    // round, 8-way bank conflicts)
    const int local = gtid % CI, sub = gtid / CI;
    T* buf = reinterpret_cast<T*>(smem + L::off_buf + g * L::buf_bytes);
    T* sgeo = reinterpret_cast<T*>(smem + L::off_geo + g * L::geo_bytes);  // P2: [6][CI]
    const T wsum = A::from(a.wsum);
    int q = 0, ntok = 0;  // chunks before this block; token waits so far
    for (int j = 0;; ++j) {
      if (!mbar_wait(&bars[kBarBlkFull + (j & 1)], (uint32_t)((j >> 1) & 1), a.wait_limit)) failed = true;
      if (named_sync_or<1, kConsumers>(failed)) { failed = true; break; }
      const BlockDesc d = sblk[j & 1];
      mbar_arrive(&bars[kBarBlkEmpty + (j & 1)]);
      if (d.nchunks < 0) break;
      const int n = d.nchunks;
      for (int i = tid; i < kAccMax; i += kConsumers) acc[i] = A::zero();
      named_sync<1, kConsumers>();  // zeroed before any phase 2

      for (int c = ((g - q) % kGroups + kGroups) % kGroups; c < n; c += kGroups) {
        const int qq = q + c;
        // ---- phase 1: element matrices of chunk c from its staged record
        if (!failed && !mbar_wait(&bars[kBarRecFull + qq % NS], (uint32_t)((qq / NS) & 1), a.wait_limit)) failed = true;
        int w_beg = 0, w_end = 0;  // this warp's contribution words (read before the record is released)
        if (!failed) {
          w_beg = desc_of(qq)->warp_off[gwarp];
          w_end = desc_of(qq)->warp_off[gwarp + 1];
        }
        // the staged vertices of chunk c and the local vertex indices of item `it`
        auto staged_verts = [&]() {
          const unsigned char* rb = stage_of(qq);
          const int n4 = (min(CI, d.item_count - c * CI) + 3) & ~3, nn = desc_of(qq)->n_nodes;
          const unsigned char* v0 = rb + sizeof(ChunkDesc) + 12 * n4;
          return StagedVerts{reinterpret_cast<const float4*>(v0), reinterpret_cast<const float4*>(v0 + 16 * nn),
                             reinterpret_cast<const float*>(v0 + 32 * nn)};
        };
        auto item_lconn = [&](int it) {
          const unsigned char* rb = stage_of(qq);
          const int n4 = (min(CI, d.item_count - c * CI) + 3) & ~3;
          return reinterpret_cast<const ushort4*>(rb + sizeof(ChunkDesc) + 4 * n4)[it];
        };
        // geometry and coefficient of item `it` of chunk c (from the staged
        // record).  A near-degenerate element (det_cancels) gets its geometry in
        // FP64 here unless `defer` is set (the P1 stiffness sends it down its own
        // rare path); returns whether it is one.
        auto item_geometry = [&](int it, Cof<T>& f, T& coef, double& coef_d, bool defer, float* c0 = nullptr) {
          const unsigned char* rb = stage_of(qq);
          const int rk = reinterpret_cast<const int32_t*>(rb + sizeof(ChunkDesc))[it];
          coef_d = a.coeff ? __ldg(a.coeff + rk) : a.cconst;  // latency covered by the geometry
          const ushort4 lc = item_lconn(it);
          const StagedVerts sv = staged_verts();
          const bool need = geometry_staged_lazy<MODE>(sv, lc, f, c0);
          if constexpr (MODE != kF64) {
            // entered only when a lane of the warp needs it
            if (!defer && __any_sync(__activemask(), need)) {
              if (need) f = staged_geometry_fp64<T>(sv, lc);
            }
          }
          coef = A::from(coef_d);
          // NaN / Inf coefficient: recorded for mg_plan_status (checked after the
          // geometry, where the load has long landed)
          if (((__double_as_longlong(coef_d) >> 52) & 0x7ff) == 0x7ff) atomicOr(&a.counters[4], 1u);
          return need;
        };
        // double-word range of an element's scale factors, recorded for mg_plan_status
        auto check_scale = [&](const T& x, const T& y) {
          if constexpr (MODE == kDW)
            if (!dw_scale_ok(x) || !dw_scale_ok(y)) atomicOr(&a.counters[4], 2u);
        };
        // P2 in the FP64 modes: the double-word geometry is worth computing once per
        // item; FP32 recomputes it in each of the item's threads (no extra barrier)
        constexpr bool kGeoOnce = ORDER == 2 && MODE != kF32;
        if (ORDER == 2 && !kGeoOnce) {
          if (!failed && c * CI + local < d.item_count) {
            Cof<T> f;
            T coef;
            double coef_d;
            item_geometry(local, f, coef, coef_d, false);
            if (a.stiff) {
              T gm[6];
              metric<T>(f, coef / f.det, gm);
              for (int u = sub; u < NU; u += TPI) buf[u * CI + local] = metric_dot<T>(gm, tab, NU, u);
            } else {
              const T sc = coef * f.det;
              for (int u = sub; u < NU; u += TPI) buf[u * CI + local] = sc * tab[6 * NU + u];
            }
          }
        } else if (ORDER == 1) {
          if (!failed && c * CI + local < d.item_count) {
            Cof<T> f;
            T coef;
            double coef_d;
            float c0[3];  // FP32 stiffness: C_0 from the edge columns (geometry_staged_lazy)
            const bool degenerate =
                item_geometry(local, f, coef, coef_d, a.stiff != 0, MODE == kF32 && a.stiff ? c0 : nullptr);
            T K[10];
            if (a.stiff) {
              // the rare elements (p1_class, or a cancelling determinant) go out of
              // line, entered only when a lane of the warp has one; that path
              // writes its entries itself
              const bool rare = degenerate || p1_class<T>(f) != kP1Common;
              // entered only when a lane of the warp has one (~0.01 % of the elements)
              if (__any_sync(__activemask(), rare)) {
                if (rare) {
                  const RareK<T> rk =
                      staged_rare_stiffness<MODE>(staged_verts(), item_lconn(local), coef_d, a.wsum, &a.counters[4]);
#pragma unroll
                  for (int u = 0; u < 10; ++u) K[u] = rk.K[u];
                }
              }
              if (rare) {
              } else if constexpr (MODE == kF32) {
                // FP32: C_0 from the face opposite vertex 0, every element
                p1_stiff_direct<T>(f, c0, coef * wsum / f.det, K);
              } else {
                const T sc = coef * wsum / f.det;
                p1_stiff_unique<T>(f, sc, K);
                check_scale(sc, K[4]);
              }
            } else {
              const T sc = coef * f.det;
              check_scale(sc, sc);
#pragma unroll
              for (int u = 0; u < 10; ++u) K[u] = sc * tab[6 * NU + u];
            }
#pragma unroll
            for (int u = 0; u < 10; ++u) buf[u * CI + local] = K[u];
          }
        } else {
          // P2: the first warp of the group computes each item's scale factors
          // once (6 metric coefficients, or coef * det for the mass); then every
          // thread forms its share of the item's 55 entries
          if (!failed && gwarp == 0 && c * CI + lane < d.item_count) {
            Cof<T> f;
            T coef;
            double coef_d;
            item_geometry(lane, f, coef, coef_d, false);
            if (a.stiff) {
              T gm[6];
              const T sc = coef / f.det;
              metric<T>(f, sc, gm);
              check_scale(sc, gm[0]);
#pragma unroll
              for (int k = 0; k < 6; ++k) sgeo[k * CI + lane] = gm[k];
            } else {
              const T sc = coef * f.det;
              check_scale(sc, sc);
              sgeo[lane] = sc;
            }
          }
          failed = group_sync_or(g, failed);
          if (!failed && c * CI + local < d.item_count) {
            if (a.stiff) {
              T gm[6];
#pragma unroll
              for (int k = 0; k < 6; ++k) gm[k] = sgeo[k * CI + local];
              for (int u = sub; u < NU; u += TPI) buf[u * CI + local] = metric_dot<T>(gm, tab, NU, u);
            } else {
              const T sc = sgeo[local];
              for (int u = sub; u < NU; u += TPI) buf[u * CI + local] = sc * tab[6 * NU + u];
            }
          }
        }
        failed = group_sync_or(g, failed);
        if (gtid == 0) mbar_arrive(&bars[kBarRecEmpty + qq % NS]);
        // ---- phase 2: segmented sums into owned slots.  Pieces of PW words of
        // one slot are summed in registers and update the slot once; within a
        // chunk every slot belongs to one thread, and the token orders the
        // chunks.
        if (!failed &&
            !mbar_wait(&bars[kBarEntFull + qq % kWordStages], (uint32_t)((qq / kWordStages) & 1), a.wait_limit))
          failed = true;
        if (c >= 1) {
          if (!failed && !mbar_wait(&bars[kBarToken + g], (uint32_t)(ntok & 1), a.wait_limit)) failed = true;
          ++ntok;
        }
        if (!failed) {
          // 8-byte pieces, [piece][lane] per warp (layout at piece_srcs)
          const int K = (w_end - w_beg) / 64;
          const uint2* ew = reinterpret_cast<const uint2*>(sent + (qq % kWordStages) * went + w_beg) + lane;
#pragma unroll 2
          for (int k = 0; k < K; ++k) {
            const uint2 pc = ew[k * 32];
            uint32_t slot;
            T v;
            if constexpr (ORDER == 1) {
              slot = (pc.y >> (kP1SlotShift - 32)) & kSlotMask;
              v = buf[pc.x & kP1SrcMask];
              A::sum_into(v, buf[(pc.x >> kP1SrcBits) & kP1SrcMask]);
              A::sum_into(v, buf[((pc.x >> (2 * kP1SrcBits)) | (pc.y << (32 - 2 * kP1SrcBits))) & kP1SrcMask]);
              A::sum_into(v, buf[(pc.y >> (3 * kP1SrcBits - 32)) & kP1SrcMask]);
            } else {
              slot = (pc.x >> kSrcBits) & kSlotMask;
              v = buf[pc.x & kSrcMask];
              A::sum_into(v, buf[pc.y & kSrcMask]);
            }
            T a = acc[slot];
            A::sum_into(a, v);
            acc[slot] = a;
          }
        }
        if (c + 1 < n) mbar_arrive(&bars[kBarToken + (g + 1) % kGroups]);  // release: the updates above precede
        failed = group_sync_or(g, failed);
        if (gtid == 0) mbar_arrive(&bars[kBarEntEmpty + qq % kWordStages]);
      }
      q += n;
      if (!failed && !mbar_wait(&bars[kBarMetaFull], (uint32_t)(j & 1), a.wait_limit)) failed = true;
      if (named_sync_or<1, kConsumers>(failed)) { failed = true; break; }
      // ---- write the owned rows, one row per thread: the stores of a pass go
      // to 32 rows at once, the accumulator reads (consecutive rows) spread
      // over the banks
      using Out = typename A::Out;
      Out* out = reinterpret_cast<Out*>(a.values);
      const int2* sm = smeta + (d.row_begin & 1);  // sm[i]: row i of the block
      for (int r = tid; r - tid < d.row_count; r += kConsumers) {
        int base = 0, len = 0, off = 0;
        if (r < d.row_count) {
          const int2 m = sm[r];
          base = m.x;
          off = m.y;
          len = ((r + 1 < d.row_count) ? sm[r + 1].x : d.acc_used) - base;
        }
        const int maxlen = __reduce_max_sync(0xffffffffu, len);
        Out* o = out + base + off;
        const T* s0 = acc + base;
#pragma unroll 4
        for (int k = 0; k < maxlen; ++k)
          if (k < len) o[k] = A::out(s0[k]);
      }
      named_sync<1, kConsumers>();
      if (tid == 0) mbar_arrive(&bars[kBarMetaEmpty]);
    }
  }
  if (failed && (tid == 0 || tid == kConsumers)) {
    atomicExch(&a.counters[2], (uint32_t)kDevErrTimeout);
    atomicExch(&a.counters[3], (uint32_t)blockIdx.x);
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&a.counters[1], 1u) == gridDim.x - 1) {
      a.counters[0] = 0;
      a.counters[1] = 0;
      __threadfence();
    }
  }
}

// Per kernel instantiation and device: SM count, opt-in shared-memory limit and
// the dynamic shared-memory size the kernel attribute has been raised to
// (only ever raised, so plans of different sizes and threads can share it).
struct KernelLaunchCache {
  static constexpr int kMaxDevices = 64;
  std::mutex mu;
  int sms[kMaxDevices] = {};
  int max_smem[kMaxDevices] = {};
  size_t attr_smem[kMaxDevices] = {};
};

template <int ORDER, int MODE>
static mg_status launch_assemble_t(AsmArgs a, cudaStream_t st)
{
  using L = AsmLayout<ORDER, MODE>;
  const size_t smem = L::total(a.ent_cap, a.stage_cap);
  static KernelLaunchCache cache;
  int dev = 0, sms = 0, per_sm = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= KernelLaunchCache::kMaxDevices) return set_error(MG_ERR_UNSUPPORTED, "device index above 63");
  {
    std::lock_guard<std::mutex> lock(cache.mu);
    if (!cache.sms[dev]) {
      MG_CUDA(cudaDeviceGetAttribute(&cache.sms[dev], cudaDevAttrMultiProcessorCount, dev));
      MG_CUDA(cudaDeviceGetAttribute(&cache.max_smem[dev], cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    }
    if (smem > (size_t)cache.max_smem[dev])
      return set_error(MG_ERR_SIZE, "assembly CTA needs " + std::to_string(smem) + " bytes of shared memory, above " +
                                        std::to_string(cache.max_smem[dev]) + " (chunks touch too many vertices)");
    if (cache.attr_smem[dev] < smem) {
      MG_CUDA(cudaFuncSetAttribute(k_assemble<ORDER, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      cache.attr_smem[dev] = smem;
    }
    sms = cache.sms[dev];
  }
  constexpr int threads = AsmShape<MODE>::threads;
  MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_assemble<ORDER, MODE>, threads, smem));
  if (per_sm < 1) return set_error(MG_ERR_SIZE, "assembly CTA does not fit on an SM (shared memory or registers)");
  const int grid = std::max(1, std::min(a.nblocks, per_sm * sms));
  if (a.nblocks > 0) k_assemble<ORDER, MODE><<<grid, threads, smem, st>>>(a);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// The coefficient in the plan's Morton element order: a chunk's items are
// consecutive ranks of one block, so the assembly reads it in runs (its elements
// are neighbours; the caller's element order may be arbitrary).
__global__ void __launch_bounds__(256) k_coeff_morton(int64_t n_elem, const int32_t* __restrict__ elem_order,
                                                      const double* __restrict__ coeff, double* __restrict__ out)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < n_elem) out[r] = __ldg(coeff + elem_order[r]);
}

mg_status launch_assemble(mg_plan* p, int op, const double* d_coeff, double c, int quad, int prec,
                          void* d_values, cudaStream_t st)
{
  if (op < MG_OP_STIFF_KAPPA || op > MG_OP_MASS_COEFF)
    return set_error(MG_ERR_INVALID_ARG, "unknown operator " + std::to_string(op));
  if (!prec_valid(prec)) return set_error(MG_ERR_INVALID_ARG, "prec must be MG_F64, MG_F32 or MG_F64_NATIVE");
  const bool needs_coeff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_MASS_COEFF);
  if (needs_coeff && !d_coeff && p->mesh->n_elem > 0)
    return set_error(MG_ERR_INVALID_ARG, "this operator needs the per-element coefficient array");
  const RefTables* t = nullptr;
  const double* d_tab = nullptr;
  MG_TRY(plan_tables(p, quad, &t, &d_tab));  // validates quad
  if (p->nnz == 0) return MG_OK;  // empty mesh: nothing to write
  if (!d_values) return set_error(MG_ERR_INVALID_ARG, "mg_assemble: null values");
  MG_TRY(plan_device(p));
  mg_mesh* m = p->mesh;
  AsmArgs a;
  a.blocks = p->d_blocks;
  a.chunk_data = p->d_chunk_data;
  a.chunk_rec = p->d_chunk_rec;
  a.chunk_wb = p->d_chunk_wb;
  a.entries = p->d_entries;
  a.row_meta = p->d_row_meta;
  a.coeff = nullptr;
  if (needs_coeff) {
    {
      std::lock_guard<std::mutex> lock(p->upload_mu);
      if (!p->d_coeff_m) MG_CUDA(cudaMalloc(&p->d_coeff_m, sizeof(double) * m->n_elem));
    }
    k_coeff_morton<<<(unsigned)((m->n_elem + 255) / 256), 256, 0, st>>>(m->n_elem, p->d_elem_order, d_coeff,
                                                                        p->d_coeff_m);
    MG_CUDA(cudaGetLastError());
    a.coeff = p->d_coeff_m;
  }
  a.cconst = op == MG_OP_STIFF_CONST ? c : 1.0;
  a.tables = d_tab;
  a.wsum = t->wsum;
  a.values = d_values;
  a.counters = p->d_counters;
  a.nblocks = p->nblocks;
  a.stiff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_STIFF_CONST);
  a.ent_cap = (int)((p->max_chunk_entries + 3) / 4 * 4);
  a.stage_cap = std::max(p->max_rec_bytes, 64);
  a.wait_limit = p->wait_limit;
  if (m->order == 1) {
    if (prec == MG_F32) return launch_assemble_t<1, kF32>(a, st);
    return prec == MG_F64_NATIVE ? launch_assemble_t<1, kF64>(a, st) : launch_assemble_t<1, kDW>(a, st);
  }
  if (prec == MG_F32) return launch_assemble_t<2, kF32>(a, st);
  return prec == MG_F64_NATIVE ? launch_assemble_t<2, kF64>(a, st) : launch_assemble_t<2, kDW>(a, st);
}

// --------------------------------------------------------------- Dirichlet --
template <typename V>
__global__ void k_dirichlet(int64_t ndof, const int32_t* rowptr, const int32_t* colind, const uint8_t* mask,
                            V* values, double* b)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= ndof) return;
  const bool mr = mask[r] != 0;
  for (int s = rowptr[r]; s < rowptr[r + 1]; ++s) {
    const int c = colind[s];
    if (mr) values[s] = (c == r) ? V(1) : V(0);
    else if (mask[c]) values[s] = V(0);
  }
  if (b && mr) b[r] = 0.0;
}

// ----------------------------------------------------------------- adjoint --
// grad_e = -sum_{i,j} lambda[dof_j] Khat_ij u[dof_i], Khat the kappa = 1
// stiffness of element e (symmetric, rows summing to zero).  Because of the
// zero row sums the form only sees differences to the element's first vertex:
// grad_e = -sum_{i,j >= 1} (lambda_j - lambda_0) Khat_ij (u_i - u_0), which removes
// the cancellation of a smooth field against the stiffness.  The differences
// are FP64 (exact for nearby values); each group (u or lambda) is rescaled by
// the power of two of its largest difference, so the double-word arithmetic on
// the FP32 pipes sees values near 1 whatever the scale of u and lambda, and the
// result is scaled back in FP64.

// biased FP64 exponent
__device__ __forceinline__ int dexp(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7ff); }

// v * 2^(1023 - emax) as a double-word value, by exponent arithmetic (emax = the
// largest biased exponent of the group, a normal number).  Parts more than 2^-74
// below the largest are dropped (a relative 2^-74 of the group).
__device__ __forceinline__ ff ff_rescaled(double v, int emax)
{
  const long long b = __double_as_longlong(v);
  if (dexp(v) + 74 < emax) return ff{0.0f, 0.0f};
  return ff_from_double_bits(__longlong_as_double(b - ((long long)(emax - 1023) << 52)));
}

// v * 2^k for |k| <= 2044 (two exact power-of-two products unless the result
// leaves the FP64 range); out of line, like the other rare FP64 paths
__device__ __noinline__ double scale_pow2(double v, int k)
{
  const int k1 = k / 2, k2 = k - k1;
  return v * __longlong_as_double((long long)(k1 + 1023) << 52) * __longlong_as_double((long long)(k2 + 1023) << 52);
}

// a * 2^k as a double: scaled on the floats when the result stays well inside
// the normal-float range (then one FP64 addition), else in FP64
__device__ __forceinline__ double ff_to_double_pow2(ff a, int k)
{
  if (a.hi == 0.0f) return 0.0;
  const int ex = (int)((__float_as_uint(a.hi) >> 23) & 0xffu) - 127 + k;
  if (k >= -100 && k <= 100 && ex >= -90 && ex <= 100) {
    const float fs = __uint_as_float((uint32_t)(k + 127) << 23);
    return ff_to_double_bits(ff{a.hi * fs, a.lo * fs});
  }
  return scale_pow2(ff_to_double_bits(a), k);
}

// Element geometry cache: the double-word Jacobian determinant and cofactors of
// every element (from the exact three-float node coordinates), written once per
// plan in the Morton order p, structure of arrays (coalesced for the kernels
// that read them: load vector, adjoint).
template <int NB>
__global__ void __launch_bounds__(256) k_elem_geometry(int64_t n_elem, const int32_t* dofs_m, GeoPtrs geo,
                                                       float2* det, float2* cof)
{
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_elem) return;
  const int32_t* d = dofs_m + p * NB;
  const int4 n = NB == 4 ? reinterpret_cast<const int4*>(dofs_m)[p] : make_int4(d[0], d[1], d[2], d[3]);
  Cof<ff> f;
  geometry_abs(geo, n, f);
  det[p] = make_float2(f.det.hi, f.det.lo);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) cof[(3 * r + c) * n_elem + p] = make_float2(f.c[r][c].hi, f.c[r][c].lo);
}

__device__ __forceinline__ void cached_geometry(const float2* det, const float2* cof, int64_t n_elem, int64_t p,
                                                Cof<ff>& f)
{
  const float2 d = det[p];
  f.det = ff{d.x, d.y};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 v = cof[(3 * r + c) * n_elem + p];
      f.c[r][c] = ff{v.x, v.y};
    }
}

// Elements are visited along a Morton curve of their centroids (elem_order,
// dofs_m = their dofs in that order), so neighbouring threads gather
// neighbouring dof values.
template <int ORDER>
__global__ void __launch_bounds__(256) k_adjoint(int64_t n_elem, const int32_t* elem_order, const int32_t* dofs_m,
                                                 const float2* gdet, const float2* gcof, const double* tables,
                                                 double wsum, const double* u, const double* lam, double* grad)
{
  constexpr int NB = ORDER == 1 ? 4 : 10, NU = ORDER == 1 ? 10 : 55;
  __shared__ ff tab[6 * NU];
  for (int i = threadIdx.x; i < 6 * NU; i += blockDim.x) tab[i] = ff_from_double(tables[i]);
  __syncthreads();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_elem) return;
  const int64_t e = elem_order[i];
  const int32_t* dofs = dofs_m + i * NB;  // this element's dofs; the first four are its vertices
  const int4 n = ORDER == 1 ? reinterpret_cast<const int4*>(dofs_m)[i] : make_int4(dofs[0], dofs[1], dofs[2], dofs[3]);
  // FP64 differences to the first dof and the largest exponent of each group
  double du[NB - 1], dl[NB - 1];
  int eu = 0, el = 0;
  {
    const double u0 = u[n.x], l0 = lam[n.x];
#pragma unroll
    for (int k = 1; k < NB; ++k) {
      const int dof = ORDER == 1 ? (k == 1 ? n.y : k == 2 ? n.z : n.w) : dofs[k];
      du[k - 1] = u[dof] - u0;
      dl[k - 1] = lam[dof] - l0;
      eu = max(eu, dexp(du[k - 1]));
      el = max(el, dexp(dl[k - 1]));
    }
  }
  if (eu == 0x7ff || el == 0x7ff) {  // Inf or NaN among u, lambda
    grad[e] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  if (eu == 0 || el == 0) {  // constant (or denormal-scale) u or lambda on the element
    grad[e] = -0.0;
    return;
  }
  Cof<ff> f;
  cached_geometry(gdet, gcof, n_elem, i, f);
  ff s = ff_make(0.0f);
  if (ORDER == 1) {
    // lambda^T K u = (wsum / det) (sum_b dl_b C_b) . (sum_b du_b C_b), C_b the cofactor columns
    ff gu[3], gl[3];
    for (int r = 0; r < 3; ++r) gu[r] = gl[r] = ff_make(0.0f);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const ff a = ff_rescaled(du[b], eu);
      const ff c = ff_rescaled(dl[b], el);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        gu[r] = gu[r] + a * f.c[r][b];
        gl[r] = gl[r] + c * f.c[r][b];
      }
    }
    s = ff_dot3(gl, gu) * (ff_from_double_bits(wsum) / f.det);
  } else {
    ff ue[NB - 1], le[NB - 1];
#pragma unroll
    for (int k = 0; k < NB - 1; ++k) {
      ue[k] = ff_rescaled(du[k], eu);
      le[k] = ff_rescaled(dl[k], el);
    }
    ff g[6];
    metric<ff>(f, ff_make(1.0f) / f.det, g);
#pragma unroll
    for (int a = 1; a < NB; ++a) {
      ff row = ff_make(0.0f);
#pragma unroll
      for (int b = 1; b < NB; ++b) {
        const int uidx = sym_index(a, b, NB);
        ff v = g[0] * tab[uidx];
#pragma unroll
        for (int p = 1; p < 6; ++p) v = v + g[p] * tab[p * NU + uidx];
        row = row + le[b - 1] * v;
      }
      s = s + row * ue[a - 1];
    }
  }
  grad[e] = -ff_to_double_pow2(s, (eu - 1023) + (el - 1023));
}

// ------------------------------------------------------------- load vector --
// b_i = sum_e s_e int_e f_h phi_i with f_h = sum_k f_k phi_k (f = 1 without a
// field): the reference's vector builder (fnEL3dA / fnEL3dB under
// traitsVectorBuilder) as two deterministic passes.
// Pass 1, one thread per element along the Morton order (position p): the
// element vector y[p nb + l] = s_e det_e sum_k Mhat_lk f_k, Mhat the reference
// mass table of the quadrature card.  Double-word arithmetic; s_e and the f_k
// are rescaled by powers of two (their largest exponents), so the result keeps
// FP64 accuracy at any scale, and is written as an IEEE double.
template <int ORDER>
__global__ void __launch_bounds__(256) k_rhs_elem(int64_t n_elem, const int32_t* elem_order, const int32_t* dofs_m,
                                                  const float2* gdet, const double* mass, const double* field,
                                                  const double* scale, double* y)
{
  constexpr int NB = ORDER == 1 ? 4 : 10, NU = ORDER == 1 ? 10 : 55;
  __shared__ ff tab[NU];
  __shared__ ff rsum[NB];
  for (int i = threadIdx.x; i < NU; i += blockDim.x) tab[i] = ff_from_double(mass[i]);
  if (threadIdx.x < NB) {
    double r = 0.0;
    for (int j = 0; j < NB; ++j) r += mass[sym_index((int)threadIdx.x, j, NB)];
    rsum[threadIdx.x] = ff_from_double(r);
  }
  __syncthreads();
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_elem) return;
  const int32_t* dofs = dofs_m + p * NB;
  const double sd = scale ? scale[elem_order[p]] : 1.0;
  const int es = dexp(sd);
  double f[NB];
  int ef = 1023;  // exponent of 1 without a field
  if (field) {
    ef = 0;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      f[k] = field[dofs[k]];
      ef = max(ef, dexp(f[k]));
    }
  }
  double2* out = reinterpret_cast<double2*>(y + p * NB);
  if (es == 0x7ff || ef == 0x7ff || es == 0 || ef == 0) {
    // Inf / NaN in s or f: NaN; zero (or denormal-scale) s or f: zero
    const double v = (es == 0x7ff || ef == 0x7ff) ? __longlong_as_double(0x7ff8000000000000ll) : 0.0;
#pragma unroll
    for (int l = 0; l < NB / 2; ++l) out[l] = make_double2(v, v);
    return;
  }
  const float2 dt = gdet[p];
  const ff sdet = ff_rescaled(sd, es) * ff{dt.x, dt.y};
  ff v[NB];
  if (field) {
    ff fr[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) fr[k] = ff_rescaled(f[k], ef);
#pragma unroll
    for (int l = 0; l < NB; ++l) {
      ff a = tab[sym_index(l, 0, NB)] * fr[0];
#pragma unroll
      for (int k = 1; k < NB; ++k) a = a + tab[sym_index(l, k, NB)] * fr[k];
      v[l] = a * sdet;
    }
  } else {
#pragma unroll
    for (int l = 0; l < NB; ++l) v[l] = rsum[l] * sdet;
  }
  // back to the true scale 2^k2
  const int k2 = (es - 1023) + (ef - 1023);
#pragma unroll
  for (int l = 0; l < NB / 2; ++l)
    out[l] = make_double2(ff_to_double_pow2(v[2 * l], k2), ff_to_double_pow2(v[2 * l + 1], k2));
}

// Pass 2, G lanes per dof: b_i = the FP64 sum of its element-vector entries,
// each lane over every G-th entry in ascending slot order, the lanes combined
// by xor shuffles in a fixed tree (bitwise reproducible, no atomics).
template <int G, int U>
__global__ void __launch_bounds__(256) k_rhs_gather(int64_t ndof, const int32_t* __restrict__ ptr,
                                                    const int32_t* __restrict__ slot, const double* __restrict__ y,
                                                    double* __restrict__ b)
{
  const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x & (G - 1);
  if (i >= ndof) return;  // whole groups: G divides the block
  const int s0 = __ldg(ptr + i), s1 = __ldg(ptr + i + 1);
  double acc = 0.0;
  for (int base = s0 + lane; base < s1; base += G * U) {
    int q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) q[u] = base + u * G < s1 ? __ldg(slot + base + u * G) : -1;
    double t[U];
#pragma unroll
    for (int u = 0; u < U; ++u) t[u] = q[u] >= 0 ? __ldg(y + q[u]) : 0.0;
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (q[u] >= 0) acc += t[u];
  }
  if constexpr (G > 1) {
    const unsigned mask = ((1u << G) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) acc += __shfl_xor_sync(mask, acc, off, G);
  }
  if (lane == 0) b[i] = acc;
}

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_assemble(mg_plan* plan, int32_t op, const double* d_coeff, double c, int32_t quad, int32_t prec,
                      void* d_values, void* stream)
{
  NvtxRange nvtx_range("mg_assemble");
  if (!plan) return set_error(MG_ERR_INVALID_ARG, "mg_assemble: null plan");
  return launch_assemble(plan, op, d_coeff, c, quad, prec, d_values, (cudaStream_t)stream);
}

mg_status mg_plan_status(mg_plan* p)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_plan_status: null plan");
  if (!p->on_device) return MG_OK;
  MG_CUDA(cudaDeviceSynchronize());
  uint32_t c[5];
  MG_CUDA(cudaMemcpy(c, p->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
  if (c[2] || c[4]) {
    const uint32_t zero[3] = {0u, 0u, 0u};
    MG_CUDA(cudaMemcpy(p->d_counters + 2, zero, sizeof(zero), cudaMemcpyHostToDevice));
  }
  if (c[2])
    return set_error(MG_ERR_CUDA, "assembly kernel: a bulk-copy wait timed out in CTA " + std::to_string(c[3]) +
                                      "; the values of that call are incomplete");
  if (c[4] & 1u)
    return set_error(MG_ERR_INVALID_ARG, "assembly: the coefficient array holds NaN or Inf (the values are not usable)");
  if (c[4] & 2u)
    return set_error(MG_ERR_UNSUPPORTED,
                     "assembly: element-matrix scales outside 2^-96 .. 2^112, where the double-word MG_F64 "
                     "assembly keeps 1e-12 accuracy; use MG_F64_NATIVE or rescale the coefficient by a power of two");
  return MG_OK;
}

mg_status mg_plan_set_wait_limit(mg_plan* p, uint32_t polls)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_plan_set_wait_limit: null plan");
  p->wait_limit = polls;
  return MG_OK;
}

mg_status mg_assemble_host(mg_plan* p, int32_t op, const double* h_coeff, double c, int32_t quad, int32_t prec,
                           void* h_values, void* stream)
{
  NvtxRange nvtx_range("mg_assemble_host");
  if (!p || (!h_values && p->nnz > 0)) return set_error(MG_ERR_INVALID_ARG, "mg_assemble_host: null argument");
  MG_TRY(plan_device(p));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t vbytes = (size_t)p->nnz * (prec_is_f64(prec) ? 8 : 4);
  if (p->tmp_values_bytes < vbytes) {
    cudaFree(p->d_tmp_values);
    p->d_tmp_values = nullptr;
    p->tmp_values_bytes = 0;
    MG_CUDA(cudaMalloc(&p->d_tmp_values, vbytes));
    p->tmp_values_bytes = vbytes;
  }
  const double* d_coeff = nullptr;
  if (h_coeff) {
    const size_t cbytes = sizeof(double) * (size_t)p->mesh->n_elem;
    if (p->tmp_coeff_bytes < cbytes) {
      cudaFree(p->d_tmp_coeff);
      p->d_tmp_coeff = nullptr;
      p->tmp_coeff_bytes = 0;
      MG_CUDA(cudaMalloc(&p->d_tmp_coeff, cbytes));
      p->tmp_coeff_bytes = cbytes;
    }
    MG_CUDA(cudaMemcpyAsync(p->d_tmp_coeff, h_coeff, cbytes, cudaMemcpyHostToDevice, st));
    d_coeff = p->d_tmp_coeff;
  }
  MG_TRY(launch_assemble(p, op, d_coeff, c, quad, prec, p->d_tmp_values, st));
  if (vbytes) MG_CUDA(cudaMemcpyAsync(h_values, p->d_tmp_values, vbytes, cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  return mg_plan_status(p);
}

mg_status mg_apply_dirichlet(mg_plan* p, const uint8_t* d_mask, int32_t prec, void* d_values, double* d_b,
                             void* stream)
{
  NvtxRange nvtx_range("mg_apply_dirichlet");
  if (!p || !d_mask || !d_values) return set_error(MG_ERR_INVALID_ARG, "mg_apply_dirichlet: null argument");
  if (!prec_valid(prec)) return set_error(MG_ERR_INVALID_ARG, "bad precision");
  MG_TRY(plan_device(p));
  const int threads = 256;
  const int blocks = (int)((p->ndof + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (blocks > 0) {
    if (prec_is_f64(prec))
      k_dirichlet<double><<<blocks, threads, 0, st>>>(p->ndof, p->d_rowptr, p->d_colind, d_mask, (double*)d_values,
                                                      d_b);
    else
      k_dirichlet<float><<<blocks, threads, 0, st>>>(p->ndof, p->d_rowptr, p->d_colind, d_mask, (float*)d_values,
                                                     d_b);
  }
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// The element geometry cache (once per plan; the mesh is immutable).  Built on
// the caller's stream and waited for, so later calls on any stream see it.
static mg_status plan_geometry(mg_plan* p, cudaStream_t st)
{
  if (p->d_geo_det) return MG_OK;
  mg_mesh* m = p->mesh;
  const int64_t E = m->n_elem;
  if (E == 0) return MG_OK;
  float2 *det = nullptr, *cof = nullptr;
  MG_CUDA(cudaMalloc(&det, sizeof(float2) * E));
  if (cudaMalloc(&cof, sizeof(float2) * 9 * E) != cudaSuccess) {
    cudaFree(det);
    return set_error(MG_ERR_ALLOC, "element geometry cache: out of device memory");
  }
  const GeoPtrs geo{m->d_xyz, m->d_node_rec, m->d_lo_z};
  const int blocks = (int)((E + 255) / 256);
  if (m->order == 1) k_elem_geometry<4><<<blocks, 256, 0, st>>>(E, p->d_dofs_morton, geo, det, cof);
  else k_elem_geometry<10><<<blocks, 256, 0, st>>>(E, p->d_dofs_morton, geo, det, cof);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFree(det);
    cudaFree(cof);
    return cuda_error(e, "element geometry cache");
  }
  p->d_geo_det = det;
  p->d_geo_cof = cof;
  return MG_OK;
}

mg_status mg_adjoint_grad(mg_plan* p, const double* d_u, const double* d_lambda, int32_t quad, double* d_grad,
                          void* stream)
{
  NvtxRange nvtx_range("mg_adjoint_grad");
  if (!p || !d_u || !d_lambda || (!d_grad && p->mesh->n_elem > 0))
    return set_error(MG_ERR_INVALID_ARG, "mg_adjoint_grad: null argument");
  const RefTables* t = nullptr;
  const double* d_tab = nullptr;
  MG_TRY(plan_tables(p, quad, &t, &d_tab));
  MG_TRY(plan_device(p));
  mg_mesh* m = p->mesh;
  const int threads = 256;
  const int blocks = (int)((m->n_elem + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  MG_TRY(plan_geometry(p, st));
  if (blocks > 0) {
    if (m->order == 1)
      k_adjoint<1><<<blocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                               p->d_geo_cof, d_tab, t->wsum, d_u, d_lambda, d_grad);
    else
      k_adjoint<2><<<blocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                               p->d_geo_cof, d_tab, t->wsum, d_u, d_lambda, d_grad);
  }
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

mg_status mg_assemble_rhs(mg_plan* p, const double* d_field, const double* d_elem_scale, int32_t quad, double* d_b,
                          void* stream)
{
  NvtxRange nvtx_range("mg_assemble_rhs");
  if (!p || (!d_b && p->ndof > 0)) return set_error(MG_ERR_INVALID_ARG, "mg_assemble_rhs: null argument");
  const RefTables* t = nullptr;
  const double* d_tab = nullptr;
  MG_TRY(plan_tables(p, quad, &t, &d_tab));  // validates quad
  if (p->ndof == 0) return MG_OK;
  MG_TRY(plan_device(p));
  MG_TRY(plan_rhs_map(p));
  mg_mesh* m = p->mesh;
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = 256;
  const int nu = m->nb * (m->nb + 1) / 2;
  MG_TRY(plan_geometry(p, st));
  const int eblocks = (int)((m->n_elem + threads - 1) / threads);
  if (eblocks > 0) {
    if (m->order == 1)
      k_rhs_elem<1><<<eblocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                                 d_tab + 6 * nu, d_field, d_elem_scale, p->d_rhs_y);
    else
      k_rhs_elem<2><<<eblocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                                 d_tab + 6 * nu, d_field, d_elem_scale, p->d_rhs_y);
    MG_CUDA(cudaGetLastError());
  }
  // two lanes per dof when dofs sum more than 16 entries on average (P1: ~24),
  // else one (P2: ~7); measured on GB300 at P1 64^3 / 128^3 and P2 48^3
  if (m->n_elem * m->nb > 16 * p->ndof)
    k_rhs_gather<2, 8><<<(int)((p->ndof * 2 + threads - 1) / threads), threads, 0, st>>>(
        p->ndof, p->d_rhs_ptr, p->d_rhs_slot, p->d_rhs_y, d_b);
  else
    k_rhs_gather<1, 8><<<(int)((p->ndof + threads - 1) / threads), threads, 0, st>>>(
        p->ndof, p->d_rhs_ptr, p->d_rhs_slot, p->d_rhs_y, d_b);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // extern "C"
