// Assembly kernels for sm_103a: element matrices of the P1/P2 bilinear forms
// reduced into CSR values, plus the Dirichlet elimination, the adjoint-gradient
// kernel and the load vector.
//
// Every element matrix is computed once, along the plan's Morton element order:
//   P1 (one pass)  k_block_asm: one CTA per block of consecutive elements, their
//                  matrices in shared memory, every diagonal or upper CSR entry
//                  summed there (the plan's block map) and written to the entry
//                  and its mirror; entries whose elements span blocks get a
//                  partial sum per block, added in block order by k_shared_sum;
//   P2 (two passes) k_elem_mat: one thread per element, its 55 unique entries to
//                  the plan's element-matrix array; k_slot_gather: one thread
//                  per diagonal or upper CSR entry, the sum of its entries in
//                  ascending Morton position (the plan's slot map).
// No atomics touch values; the per-entry summation order is fixed by the plan,
// so the results are bitwise reproducible.
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
#include <cfloat>
#include <cmath>
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

// A P1 element matrix returned by value (the out-of-line rare paths: no register
// of the caller is passed by address, so the common path keeps its registers).
template <typename T>
struct RareK {
  T K[10];
};

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

// ------------------------------------------------------------ assembly --
// P1: the one-pass block assembly (k_block_asm, k_shared_sum, below).
// P2, two passes, each element computed once:
//   k_elem_mat     one thread per element, along the plan's Morton order p: the
//                  unique entries u of its (symmetric) element matrix into the
//                  plan's element-matrix array em;
//   k_slot_gather  one thread per diagonal or upper CSR entry: the sum of the em
//                  entries of every element holding both of its dofs, in
//                  ascending p (the slot map, build_slot_map), written to the
//                  entry and to its mirror -- a fixed order, so the values are
//                  bitwise reproducible, with no atomics.

// Geometry of an element from the mesh's absolute node records, in the mode's
// arithmetic; returns whether the determinant cancels (det_cancels).
//  FP32          edges (hi_k - hi_0) + (mid_k - mid_0), to a float ulp of the
//                edge; with c0 (P1 stiffness) also C_0 = (x3 - x1) x (x2 - x1)
//                from the edge columns;
//  double-word   edges dw_diff3 of the three floats: the exact FP64 difference
//                of the mesh coordinates (the reference's x_k - x_0) to ~2^-47;
//  FP64          from the FP64 coordinates.
template <int MODE>
__device__ __forceinline__ bool geometry_abs_lazy(const GeoPtrs& g, int4 n, Cof<typename Arith<MODE>::T>& f,
                                                  float* c0)
{
  using T = typename Arith<MODE>::T;
  T J[3][3];
  if constexpr (MODE == kF64) {
    const double4_32a x0 = g.xyz[n.x];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double4_32a xk = g.xyz[k == 0 ? n.y : (k == 1 ? n.z : n.w)];
#pragma unroll
      for (int r = 0; r < 3; ++r) J[r][k] = comp(xk, r) - comp(x0, r);
    }
    cofactors<double>(J, f);
    return false;
  } else {
    const float4 a0 = g.rec[2 * (int64_t)n.x], b0 = g.rec[2 * (int64_t)n.x + 1];
    const float lz0 = MODE == kDW ? g.loz[n.x] : 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int64_t id = k == 0 ? n.y : (k == 1 ? n.z : n.w);
      const float4 ak = g.rec[2 * id], bk = g.rec[2 * id + 1];
      const float lzk = MODE == kDW ? g.loz[id] : 0.0f;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        if constexpr (MODE == kF32)
          J[r][k] = (rec_hi(ak, r) - rec_hi(a0, r)) + (rec_mid(ak, bk, r) - rec_mid(a0, b0, r));
        else
          J[r][k] = dw_diff3(rec_hi(ak, r), rec_hi(a0, r), rec_mid(ak, bk, r), rec_mid(a0, b0, r), rec_lo(bk, lzk, r),
                             rec_lo(b0, lz0, r));
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
    return det_cancels<T>(J, f);
  }
}

// Near-degenerate elements: the FP64 geometry from the mesh's FP64 coordinates,
// out of line and returned by value.
template <typename T>
static __device__ __noinline__ Cof<T> abs_geometry_fp64(const double4_32a* xyz, int4 n)
{
  Fetch<kF64> D;
  D.x[0] = xyz[n.x];
  D.x[1] = xyz[n.y];
  D.x[2] = xyz[n.z];
  D.x[3] = xyz[n.w];
  Cof<double> g;
  geometry(D, g);
  Cof<T> f;
  store_geometry(g, f);
  return f;
}

// The rare P1 stiffness elements (p1_class, or a cancelling determinant): the
// geometry in FP64 from the mesh's FP64 coordinates and C_0 from the face
// opposite vertex 0, returned by value (out of line).
template <int MODE>
static __device__ __noinline__ RareK<typename Arith<MODE>::T> abs_rare_stiffness(const double4_32a* xyz, int4 n,
                                                                                 double coef, double wsum,
                                                                                 uint32_t* flags)
{
  using T = typename Arith<MODE>::T;
  Fetch<kF64> D;
  D.x[0] = xyz[n.x];
  D.x[1] = xyz[n.y];
  D.x[2] = xyz[n.z];
  D.x[3] = xyz[n.w];
  Cof<double> d;
  geometry(D, d);
  double f2[3], f3[3], c0[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    f2[r] = comp(D.x[2], r) - comp(D.x[1], r);
    f3[r] = comp(D.x[3], r) - comp(D.x[1], r);
  }
  c0[0] = f3[1] * f2[2] - f3[2] * f2[1];
  c0[1] = f3[2] * f2[0] - f3[0] * f2[2];
  c0[2] = f3[0] * f2[1] - f3[1] * f2[0];
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

__device__ __forceinline__ void em_put(void* em, int64_t i, float v) { static_cast<float*>(em)[i] = v; }
__device__ __forceinline__ void em_put(void* em, int64_t i, ff v)
{
  static_cast<float2*>(em)[i] = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ void em_put(void* em, int64_t i, double v) { static_cast<double*>(em)[i] = v; }
template <typename T> __device__ __forceinline__ T em_get(const void* em, uint32_t i);
template <> __device__ __forceinline__ float em_get<float>(const void* em, uint32_t i)
{
  return __ldg(static_cast<const float*>(em) + i);
}
template <> __device__ __forceinline__ ff em_get<ff>(const void* em, uint32_t i)
{
  const float2 v = __ldg(static_cast<const float2*>(em) + i);
  return ff{v.x, v.y};
}
template <> __device__ __forceinline__ double em_get<double>(const void* em, uint32_t i)
{
  return __ldg(static_cast<const double*>(em) + i);
}

struct ElemArgs {
  int64_t n_elem;
  const int32_t* elem_order;  // Morton position -> element (the caller's numbering)
  const int32_t* dofs_m;      // dofs in Morton order (nb each; the first four are the vertices)
  GeoPtrs geo;
  const double* coeff;        // per element in the caller's order, or null
  double cconst;              // used when coeff is null
  const double* tables;       // unique-entry tables: stiff[6][nu] then mass[nu]
  double wsum;
  int stiff;
  void* em;                   // out: nu x n_elem entries
  uint32_t* flags;            // bit 0: NaN / Inf coefficient; bit 1: outside the double-word range
};

// The coefficient and the vertex dofs of Morton element p.
__device__ __forceinline__ double elem_coef(const ElemArgs& a, int64_t p)
{
  return a.coeff ? __ldg(a.coeff + a.elem_order[p]) : a.cconst;
}
__device__ __forceinline__ int4 elem_nodes(const ElemArgs& a, int64_t p)
{
  return __ldg(reinterpret_cast<const int4*>(a.dofs_m) + p);
}

// The P1 element matrix from the element's vertex dofs n and coefficient coef_d
// (loaded by the caller, elem_nodes / elem_coef).
template <int MODE>
__device__ __forceinline__ void p1_element(const ElemArgs& a, const typename Arith<MODE>::T* tab, int4 n,
                                           double coef_d, typename Arith<MODE>::T K[10])
{
  using A = Arith<MODE>;
  using T = typename A::T;
  constexpr int NU = 10;
  Cof<T> f;
  float c0[3];
  const bool degenerate = geometry_abs_lazy<MODE>(a.geo, n, f, MODE == kF32 && a.stiff ? c0 : nullptr);
  // NaN / Inf coefficient: recorded for mg_plan_status (checked after the
  // geometry, where the load has long landed)
  if (((__double_as_longlong(coef_d) >> 52) & 0x7ff) == 0x7ff) atomicOr(a.flags, 1u);
  const T coef = A::from(coef_d);
  if (a.stiff) {
    // the rare elements (p1_class, or a cancelling determinant) go out of line,
    // entered only when a lane of the warp has one (~0.01 % of the elements)
    const bool rare = degenerate || p1_class<T>(f) != kP1Common;
    if (__any_sync(__activemask(), rare)) {
      if (rare) {
        const RareK<T> rk = abs_rare_stiffness<MODE>(a.geo.xyz, n, coef_d, a.wsum, a.flags);
#pragma unroll
        for (int u = 0; u < 10; ++u) K[u] = rk.K[u];
      }
    }
    if (!rare) {
      const T sc = coef * A::from(a.wsum) / f.det;
      if constexpr (MODE == kF32) {
        p1_stiff_direct<T>(f, c0, sc, K);  // C_0 from the face opposite vertex 0
      } else {
        p1_stiff_unique<T>(f, sc, K);
        if constexpr (MODE == kDW)
          if (!dw_scale_ok(sc) || !dw_scale_ok(K[4])) atomicOr(a.flags, 2u);
      }
    }
  } else {
    if constexpr (MODE != kF64) {
      if (__any_sync(__activemask(), degenerate)) {
        if (degenerate) f = abs_geometry_fp64<T>(a.geo.xyz, n);
      }
    }
    const T sc = coef * f.det;
    if constexpr (MODE == kDW)
      if (!dw_scale_ok(sc)) atomicOr(a.flags, 2u);
#pragma unroll
    for (int u = 0; u < 10; ++u) K[u] = sc * tab[6 * NU + u];
  }
}

// The element pass of the two-pass P2 assembly: one thread per element along
// the plan's Morton order p, its 55 entries to em[u * E + p] (entry-major: the
// stores of one u coalesce across the warp), the metric contraction reading the
// tables from shared memory.
template <int MODE>
__global__ void __launch_bounds__(256, 1) k_elem_mat(ElemArgs a)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  constexpr int NU = 55;
  __shared__ T tab[7 * NU];
  for (int i = threadIdx.x; i < 7 * NU; i += blockDim.x) tab[i] = A::from(a.tables[i]);
  __syncthreads();
  const int64_t E = a.n_elem;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  {
    if (p >= E) return;
    const double coef_d = a.coeff ? __ldg(a.coeff + a.elem_order[p]) : a.cconst;
    const int32_t* dp = a.dofs_m + p * 10;
    const int4 n = make_int4(dp[0], dp[1], dp[2], dp[3]);
    Cof<T> f;
    const bool degenerate = geometry_abs_lazy<MODE>(a.geo, n, f, nullptr);
    if (((__double_as_longlong(coef_d) >> 52) & 0x7ff) == 0x7ff) atomicOr(a.flags, 1u);
    const T coef = A::from(coef_d);
    if constexpr (MODE != kF64) {
      if (__any_sync(__activemask(), degenerate)) {
        if (degenerate) f = abs_geometry_fp64<T>(a.geo.xyz, n);
      }
    }
    if (a.stiff) {
      T g[6];
      const T sc = coef / f.det;
      metric<T>(f, sc, g);
      if constexpr (MODE == kDW)
        if (!dw_scale_ok(sc) || !dw_scale_ok(g[0])) atomicOr(a.flags, 2u);
#pragma unroll 5
      for (int u = 0; u < NU; ++u) em_put(a.em, u * E + p, metric_dot<T>(g, tab, NU, u));
    } else {
      const T sc = coef * f.det;
      if constexpr (MODE == kDW)
        if (!dw_scale_ok(sc)) atomicOr(a.flags, 2u);
#pragma unroll 5
      for (int u = 0; u < NU; ++u) em_put(a.em, u * E + p, sc * tab[6 * NU + u]);
    }
  }
}

// One warp per group of 32 diagonal or upper CSR entries (the slot map's
// layout): lane l sums the sources src[o + 32 j + l] of its entry, j < L, in the
// slot map's order, K at a time, and writes the sum to the entry and to its
// mirror (the operators are symmetric).  Software-pipelined: the indices of the
// next K sources (one coalesced line per j) and the output positions load while
// the current element-matrix values are in flight.  Padding sources
// (kPadSource) read the zero entry `zero` past the element matrices.
template <int MODE, int K>
__global__ void __launch_bounds__(256) k_slot_gather(int64_t n_groups, int64_t n_upper, const int32_t* __restrict__ goff,
                                                     const int32_t* __restrict__ uslot,
                                                     const int32_t* __restrict__ umirror,
                                                     const uint32_t* __restrict__ src, const void* __restrict__ em,
                                                     uint32_t zero, typename Arith<MODE>::Out* __restrict__ values)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (g >= n_groups) return;
  const int lane = threadIdx.x & 31;
  const int64_t t = 32 * g + lane;
  const bool live = t < n_upper;
  const int32_t out_a = live ? __ldg(uslot + t) : 0, out_m = live ? __ldg(umirror + t) : 0;
  const int32_t o = goff[g], L = (goff[g + 1] - o) >> 5;
  const uint32_t* s = src + o + lane;
  uint32_t nxt[K];
#pragma unroll
  for (int i = 0; i < K; ++i) nxt[i] = i < L ? __ldg(s + 32 * i) : kPadSource;
  T v = A::zero();
  for (int32_t j = 0; j < L; j += K) {
    uint32_t idx[K];
#pragma unroll
    for (int i = 0; i < K; ++i) idx[i] = min(nxt[i], zero);
#pragma unroll
    for (int i = 0; i < K; ++i) nxt[i] = j + K + i < L ? __ldg(s + 32 * (j + K + i)) : kPadSource;
    T x[K];
#pragma unroll
    for (int i = 0; i < K; ++i) x[i] = j + i < L ? em_get<T>(em, idx[i]) : A::zero();
#pragma unroll
    for (int i = 0; i < K; ++i)
      if (j + i < L) A::sum_into(v, x[i]);
  }
  if (live) {
    const typename A::Out r = A::out(v);
    values[out_a] = r;
    if (out_m != out_a) values[out_m] = r;
  }
}

// ---------------------------------------------------- one-pass assembly (P1) --
// k_block_asm: one CTA per block of kElemBlock consecutive Morton positions.
//   1. each thread computes the element matrices of one or two elements into
//      shared memory (10 unique entries each);
//   2. each warp takes groups of 32 of the block's local entries (the block map):
//      lane l sums its entry's local sources in ascending p, and writes the sum
//      to the CSR entry and its mirror when every source of the entry lies in
//      this block, else to the entry's partial-sum slot.
// k_shared_sum: one warp per group of 32 shared entries: the partial sums in
//   ascending block (coalesced [j][lane]), written to the entry and its mirror.
// Each entry's summation order is fixed by the plan, so the values are bitwise
// reproducible; no atomics, no element matrix leaves the SM.
struct BlockArgs {
  const int32_t* bgrp;
  const int32_t* bsrc0;
  const int32_t* bgoff;
  const uint16_t* bsrc;
  const int2* bout;
  void* partial;  // 8-byte slots: float2 (double-word), double, or a float in the low half
};

__device__ __forceinline__ void partial_put(void* pp, int32_t q, float v) { static_cast<float2*>(pp)[q].x = v; }
__device__ __forceinline__ void partial_put(void* pp, int32_t q, ff v)
{
  static_cast<float2*>(pp)[q] = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ void partial_put(void* pp, int32_t q, double v) { static_cast<double*>(pp)[q] = v; }
template <typename T> __device__ __forceinline__ T partial_get(const void* pp, int32_t q);
template <> __device__ __forceinline__ float partial_get<float>(const void* pp, int32_t q)
{
  return __ldg(static_cast<const float2*>(pp) + q).x;
}
template <> __device__ __forceinline__ ff partial_get<ff>(const void* pp, int32_t q)
{
  const float2 v = __ldg(static_cast<const float2*>(pp) + q);
  return ff{v.x, v.y};
}
template <> __device__ __forceinline__ double partial_get<double>(const void* pp, int32_t q)
{
  return __ldg(static_cast<const double*>(pp) + q);
}

// Block-map staging in shared memory: the block's local sources (up to
// kStageSrc, the first groups' rows) and group offsets (up to kStageGroups + 1),
// copied with cp.async while the element matrices are computed.
constexpr int kStageSrc = 6144;
constexpr int kStageGroups = 96;
// dynamic shared memory of a block: its element matrices (BE x NU entries, then
// the zero of the padding sources), the staged sources and group offsets
template <typename T, int BE, int NU>
__host__ __device__ constexpr size_t block_em_bytes()
{
  return ((sizeof(T) * (BE * NU + 1) + 15) / 16) * 16;
}
template <typename T, int BE, int NU>
__host__ __device__ constexpr size_t block_smem_bytes()
{
  return block_em_bytes<T, BE, NU>() + 2 * kStageSrc + 4 * (kStageGroups + 1);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem));
}

// The block's map rows into shared memory with cp.async (waited for by the
// caller's cp.async.wait_all): whole 16-byte chunks of its local sources (group
// offsets are multiples of 32 sources, so the range is 64-byte aligned) and its
// group offsets, each up to the stage's size.
template <int THREADS>
__device__ __forceinline__ void stage_block_map(const BlockArgs& bm, int32_t g0, int32_t g1, int32_t src0,
                                                int32_t src1, uint16_t* s_src, int32_t* s_goff)
{
  const int32_t n_src = min(src1 - src0, kStageSrc), n_goff = min(g1 - g0, kStageGroups) + 1;
  for (int i = threadIdx.x; i < n_src / 8; i += THREADS) cp_async16(s_src + 8 * i, bm.bsrc + src0 + 8 * i);
  for (int i = threadIdx.x; i < n_goff; i += THREADS) cp_async4(s_goff + i, bm.bgoff + g0 + i);
  asm volatile("cp.async.commit_group;\n" ::);
}

// Phase 2 of the block assembly: each warp takes groups of 32 of the block's
// runs; lane l sums its run's sources from the element matrices em in shared
// memory (4 at a time, ascending p) and writes a complete entry to its CSR
// position and mirror, a shared entry's partial to its slot.  Rows past the
// stage come from global memory.
template <int MODE, int THREADS>
__device__ __forceinline__ void block_sums(const BlockArgs& bm, int32_t g0, int32_t g1, int32_t src0,
                                           const uint16_t* s_src, const int32_t* s_goff,
                                           const typename Arith<MODE>::T* em,
                                           typename Arith<MODE>::Out* __restrict__ values)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  const int lane = threadIdx.x & 31;
  for (int32_t g = g0 + (threadIdx.x >> 5); g < g1; g += THREADS / 32) {
    const int2 out = bm.bout[32 * g + lane];  // used after the sum: its latency overlaps it
    const int32_t gi = g - g0;
    const int32_t o = gi < kStageGroups ? s_goff[gi] : bm.bgoff[g];
    const int32_t o1 = gi + 1 <= kStageGroups ? s_goff[gi + 1] : bm.bgoff[g + 1];
    const int32_t L = (o1 - o) >> 5;
    T v = A::zero();
    if (o1 - src0 <= kStageSrc) {
      const uint16_t* s = s_src + (o - src0) + lane;
      int32_t j = 0;
      for (; j + 4 <= L; j += 4) {
        const uint32_t i0 = s[32 * j], i1 = s[32 * j + 32], i2 = s[32 * j + 64], i3 = s[32 * j + 96];
        const T x0 = em[i0], x1 = em[i1], x2 = em[i2], x3 = em[i3];
        A::sum_into(v, x0);
        A::sum_into(v, x1);
        A::sum_into(v, x2);
        A::sum_into(v, x3);
      }
      for (; j < L; ++j) A::sum_into(v, em[s[32 * j]]);
    } else {
      // past the stage (rare): the rows from global memory, 4 in flight
      const uint16_t* s = bm.bsrc + o + lane;
      int32_t j = 0;
      for (; j + 4 <= L; j += 4) {
        const uint32_t i0 = __ldg(s + 32 * j), i1 = __ldg(s + 32 * j + 32), i2 = __ldg(s + 32 * j + 64),
                       i3 = __ldg(s + 32 * j + 96);
        A::sum_into(v, em[i0]);
        A::sum_into(v, em[i1]);
        A::sum_into(v, em[i2]);
        A::sum_into(v, em[i3]);
      }
      for (; j < L; ++j) A::sum_into(v, em[__ldg(s + 32 * j)]);
    }
    if (out.x >= 0) {
      const typename A::Out r = A::out(v);
      values[out.x] = r;
      if (out.y != out.x) values[out.y] = r;
    } else if (out.x != kNoOutput) {
      partial_put(bm.partial, -1 - out.x, v);
    }
  }
}

// P1: one CTA per block of kElemBlock elements.  THREADS per CTA: 512 (one
// element each, two CTAs per SM) for the double-word and FP64 arithmetic, 256
// (two elements each, four CTAs per SM) for FP32 -- measured on GB300 at P1
// 128^3 (the double-word loop over two elements spills).
template <int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS, 2048 / THREADS / 2)
    k_block_asm(ElemArgs a, BlockArgs bm, typename Arith<MODE>::Out* __restrict__ values)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  constexpr int NU = 10;
  extern __shared__ __align__(16) unsigned char smem[];
  T* em = reinterpret_cast<T*>(smem);  // the block's element matrices, then a zero (padding source)
  uint16_t* s_src = reinterpret_cast<uint16_t*>(smem + block_em_bytes<T, kElemBlock, NU>());
  int32_t* s_goff = reinterpret_cast<int32_t*>(s_src + kStageSrc);
  __shared__ T tab[7 * NU];
  const int32_t g0 = bm.bgrp[blockIdx.x], g1 = bm.bgrp[blockIdx.x + 1];
  const int32_t src0 = bm.bsrc0[blockIdx.x], src1 = bm.bsrc0[blockIdx.x + 1];
  stage_block_map<THREADS>(bm, g0, g1, src0, src1, s_src, s_goff);
  const int64_t p0 = (int64_t)blockIdx.x * kElemBlock;
  const int64_t E = a.n_elem;
  for (int i = threadIdx.x; i < 7 * NU; i += THREADS) tab[i] = A::from(a.tables[i]);
  if (threadIdx.x == 0) em[kElemBlock * NU] = A::zero();
  __syncthreads();
#pragma unroll 1
  for (int i = 0; i < kElemBlock / THREADS; ++i) {
    const int lp = i * THREADS + threadIdx.x;
    if (p0 + lp < E) {
      T K[NU];
      p1_element<MODE>(a, tab, elem_nodes(a, p0 + lp), elem_coef(a, p0 + lp), K);
#pragma unroll
      for (int u = 0; u < NU; ++u) em[lp * NU + u] = K[u];
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  block_sums<MODE, THREADS>(bm, g0, g1, src0, s_src, s_goff, em, values);
}

template <int MODE>
__global__ void __launch_bounds__(256) k_shared_sum(int64_t n_groups, const int32_t* __restrict__ sgoff,
                                                    const int2* __restrict__ sout, const void* __restrict__ partial,
                                                    typename Arith<MODE>::Out* __restrict__ values)
{
  using A = Arith<MODE>;
  using T = typename A::T;
  const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (g >= n_groups) return;
  const int lane = threadIdx.x & 31;
  const int2 out = sout[32 * g + lane];
  const int32_t o = sgoff[g], L = (sgoff[g + 1] - o) >> 5;
  T v = A::zero();
  // 8 partials in flight, summed in ascending j
  for (int32_t j = 0; j < L; j += 8) {
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = j + i < L ? partial_get<T>(partial, o + 32 * (j + i) + lane) : A::zero();
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (j + i < L) A::sum_into(v, x[i]);
  }
  if (out.x >= 0) {
    const typename A::Out r = A::out(v);
    values[out.x] = r;
    if (out.y != out.x) values[out.y] = r;
  }
}

// Sets the dynamic shared-memory limit of a kernel once per device (the first
// assembly of each kind on a device).
template <typename K>
static mg_status allow_smem(K kernel, size_t bytes, std::once_flag (&once)[64])
{
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  cudaError_t err = cudaSuccess;
  std::call_once(once[dev & 63],
                 [&] { err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes); });
  MG_CUDA(err);
  return MG_OK;
}

template <int MODE>
static mg_status launch_block_t(mg_plan* p, const ElemArgs& a, void* d_values, cudaStream_t st)
{
  using Out = typename Arith<MODE>::Out;
  using T = typename Arith<MODE>::T;
  const BlockArgs bm{p->d_bgrp, p->d_bsrc0, p->d_bgoff, p->d_bsrc, p->d_bout, p->d_partial};
  static std::once_flag once[64];
  if (a.n_elem > 0) {
    constexpr size_t smem = block_smem_bytes<T, kElemBlock, 10>();
    constexpr int threads = MODE == kF32 ? 256 : 512;
    MG_TRY(allow_smem(k_block_asm<MODE, threads>, smem, once));
    k_block_asm<MODE, threads><<<(unsigned)p->n_blocks, threads, smem, st>>>(a, bm, static_cast<Out*>(d_values));
  }
  MG_CUDA(cudaGetLastError());
  if (p->n_sgroups > 0)
    k_shared_sum<MODE><<<(unsigned)((p->n_sgroups + 7) / 8), 256, 0, st>>>(p->n_sgroups, p->d_sgoff, p->d_sout,
                                                                         p->d_partial, static_cast<Out*>(d_values));
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// The element-matrix array of a plan (allocated by its first assembly).
static mg_status plan_gather(mg_plan* p)
{
  std::lock_guard<std::mutex> lock(p->upload_mu);
  if (!p->d_em) {
    // nunique x n_elem entries of up to 8 bytes, then one zero entry (8 bytes:
    // the FP32 gather reads its first float) for the padding sources
    const int64_t n = (int64_t)nunique(p->mesh->order) * p->mesh->n_elem;
    MG_CUDA(cudaMalloc(&p->d_em, sizeof(double) * (size_t)(n + 1)));
    MG_CUDA(cudaMemset(static_cast<double*>(p->d_em) + n, 0, sizeof(double)));
  }
  return MG_OK;
}

template <int MODE>
static mg_status launch_gather_t(mg_plan* p, const ElemArgs& a, void* d_values, cudaStream_t st)
{
  constexpr int ORDER = 2;
  const int64_t E = a.n_elem;
  if (E > 0) k_elem_mat<MODE><<<(unsigned)((E + 255) / 256), 256, 0, st>>>(a);
  MG_CUDA(cudaGetLastError());
  using Out = typename Arith<MODE>::Out;
  const unsigned blocks = (unsigned)((p->n_groups + 7) / 8);  // 8 warps (groups) per CTA
  // the zero entry: index nunique * n_elem of the 8-byte entries, 2 * that of floats
  const uint32_t zero = (uint32_t)((MODE == kF32 ? 2 : 1) * (int64_t)nunique(ORDER) * E);
  // 8 sources in flight per thread (measured on GB300 at P1 128^3 and P2 48^3
  // against 4 and 16)
  if (p->n_groups > 0)
    k_slot_gather<MODE, 8><<<blocks, 256, 0, st>>>(p->n_groups, p->n_upper, p->d_goff, p->d_uslot, p->d_umirror,
                                                   p->d_src, p->d_em, zero, static_cast<Out*>(d_values));
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

static mg_status launch_assemble_gather(mg_plan* p, int op, const double* d_coeff, double c, const RefTables* t,
                                        const double* d_tab, int prec, void* d_values, cudaStream_t st)
{
  mg_mesh* m = p->mesh;
  if (!uses_block_map(m->order)) MG_TRY(plan_gather(p));
  const bool needs_coeff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_MASS_COEFF);
  ElemArgs a;
  a.n_elem = m->n_elem;
  a.elem_order = p->d_elem_order;
  a.dofs_m = p->d_dofs_morton;
  a.geo = GeoPtrs{m->d_xyz, m->d_node_rec, m->d_lo_z};
  a.coeff = needs_coeff ? d_coeff : nullptr;
  a.cconst = op == MG_OP_STIFF_CONST ? c : 1.0;
  a.tables = d_tab;
  a.wsum = t->wsum;
  a.stiff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_STIFF_CONST);
  a.em = p->d_em;
  a.flags = p->d_counters + 4;
  if (uses_block_map(m->order)) {
    if (prec == MG_F32) return launch_block_t<kF32>(p, a, d_values, st);
    return prec == MG_F64_NATIVE ? launch_block_t<kF64>(p, a, d_values, st) : launch_block_t<kDW>(p, a, d_values, st);
  }
  if (prec == MG_F32) return launch_gather_t<kF32>(p, a, d_values, st);
  return prec == MG_F64_NATIVE ? launch_gather_t<kF64>(p, a, d_values, st) : launch_gather_t<kDW>(p, a, d_values, st);
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
  return launch_assemble_gather(p, op, d_coeff, c, t, d_tab, prec, d_values, st);
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
                                                  const double* scale, double* y, int two_valued)
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
    if (ORDER == 1 && two_valued) {
      // M^_lk = o + (d - o) [l = k]: (M^ f)_l = o sum_k f_k + (d - o) f_l, with
      // d = tab(0,0) and o = tab(0,1) from the table
      const ff o = tab[1], dmo = tab[0] - tab[1];
      ff sf = fr[0];
#pragma unroll
      for (int k = 1; k < NB; ++k) sf = sf + fr[k];
      const ff base = o * sf;
#pragma unroll
      for (int l = 0; l < NB; ++l) v[l] = (base + dmo * fr[l]) * sdet;
    } else {
#pragma unroll
      for (int l = 0; l < NB; ++l) {
        ff a = tab[sym_index(l, 0, NB)] * fr[0];
#pragma unroll
        for (int k = 1; k < NB; ++k) a = a + tab[sym_index(l, k, NB)] * fr[k];
        v[l] = a * sdet;
      }
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
  uint32_t flags = 0;
  MG_CUDA(cudaMemcpy(&flags, p->d_counters + 4, sizeof(flags), cudaMemcpyDeviceToHost));
  if (flags) {
    const uint32_t zero = 0u;
    MG_CUDA(cudaMemcpy(p->d_counters + 4, &zero, sizeof(zero), cudaMemcpyHostToDevice));
  }
  if (flags & 1u)
    return set_error(MG_ERR_INVALID_ARG, "assembly: the coefficient array holds NaN or Inf (the values are not usable)");
  if (flags & 2u)
    return set_error(MG_ERR_UNSUPPORTED,
                     "assembly: element-matrix scales outside 2^-96 .. 2^112, where the double-word MG_F64 "
                     "assembly keeps 1e-12 accuracy; use MG_F64_NATIVE or rescale the coefficient by a power of two");
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
  // A P1 mass table with one diagonal and one off-diagonal value (to a few ulps:
  // every symmetric card gives (1 + [i = j]) |T^| / 20) takes the two-value form
  // of the mat-vec in the element pass.
  int two_valued = 0;
  if (m->order == 1) {
    const double d = t->mass[0], o = t->mass[1];
    double mx = 0.0, dev = 0.0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        mx = std::max(mx, std::fabs(t->mass[4 * i + j]));
        dev = std::max(dev, std::fabs(t->mass[4 * i + j] - (i == j ? d : o)));
      }
    two_valued = dev <= 8.0 * DBL_EPSILON * mx ? 1 : 0;
  }
  if (eblocks > 0) {
    if (m->order == 1)
      k_rhs_elem<1><<<eblocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                                 d_tab + 6 * nu, d_field, d_elem_scale, p->d_rhs_y, two_valued);
    else
      k_rhs_elem<2><<<eblocks, threads, 0, st>>>(m->n_elem, p->d_elem_order, p->d_dofs_morton, p->d_geo_det,
                                                 d_tab + 6 * nu, d_field, d_elem_scale, p->d_rhs_y, 0);
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
