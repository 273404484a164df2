// Assembly kernels for sm_103a: element matrices of the P1/P2 bilinear forms
// reduced straight into CSR values, plus the Dirichlet elimination, the
// adjoint-gradient kernel and the load vector.
//
// One CTA owns one block of rows (see mg_plan.cpp).  Per chunk of elements:
//   phase 1  each element's matrix is computed into shared memory, stored
//            entry-major (buf[k * CI + item]) so that the stores are
//            bank-conflict free;
//   phase 2  every thread walks its own contribution list (coalesced 4-byte
//            words) and adds buf[src] into accumulator slot (word >> 16) * 256 +
//            threadIdx.x, a slot no other thread touches.
// After the last chunk the accumulators of each owned row are written to the
// row's contiguous CSR range.  No atomics; the per-slot summation order is the
// element order, so results are bitwise reproducible.
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
//   P1         the reference gradients are constant, so
//              K_ij = coef sum_q w_q / det (c_i . c_j) with c_1..3 = C_0..2,
//              c_0 = -(c_1 + c_2 + c_3);
//   mass       K_ij = coef det sum_q w_q phi^_i phi^_j.
// detJ is signed, as in the reference (positive on checked meshes).
#include <cstdio>

#include "mg_internal.h"

namespace mg {

struct AsmArgs {
  const BlockDesc* blocks;
  const int32_t* items;
  const int64_t* chunk_ptr;
  const uint32_t* entries;
  const int32_t* rows;
  const int32_t* row_acc;
  const int32_t* rowptr;
  const int4* conn;
  const double4_32a* xyz;
  const float4* xyz_hi;
  const float4* xyz_lo;
  const double* coeff;  // per element, or null
  double cconst;        // used when coeff is null
  const double* tables; // stiff (6 nb^2) then mass (nb^2)
  double wsum;
  void* values;
};

// Flatness threshold of the FP32 path: when |det| falls below this fraction of
// the product of the edge-vector lengths, the Jacobian is recomputed in FP64.
constexpr float kFlatTol = 1e-3f;

template <typename V>
struct Cof {
  V c[3][3];  // cofactor matrix C[r][k] of J; column a of C = J^-T e_a * det
  V det;
};

__device__ __forceinline__ void cofactors64(const double4_32a* xyz, int4 n, Cof<double>& f)
{
  const double4_32a a = xyz[n.x], b = xyz[n.y], c = xyz[n.z], d = xyz[n.w];
  const double J00 = b.x - a.x, J01 = c.x - a.x, J02 = d.x - a.x;
  const double J10 = b.y - a.y, J11 = c.y - a.y, J12 = d.y - a.y;
  const double J20 = b.z - a.z, J21 = c.z - a.z, J22 = d.z - a.z;
  f.c[0][0] = J11 * J22 - J12 * J21;
  f.c[0][1] = J12 * J20 - J10 * J22;
  f.c[0][2] = J10 * J21 - J11 * J20;
  f.c[1][0] = J02 * J21 - J01 * J22;
  f.c[1][1] = J00 * J22 - J02 * J20;
  f.c[1][2] = J01 * J20 - J00 * J21;
  f.c[2][0] = J01 * J12 - J02 * J11;
  f.c[2][1] = J02 * J10 - J00 * J12;
  f.c[2][2] = J00 * J11 - J01 * J10;
  f.det = J00 * f.c[0][0] + J01 * f.c[0][1] + J02 * f.c[0][2];
}

// FP32 geometry from the float-pair coordinates: each edge vector is
// (hi_k - hi_0) + (lo_k - lo_0), accurate to a few float ulps of the edge itself.
// Flat elements fall back to FP64 cofactors.
__device__ __forceinline__ void cofactors32(const float4* hi, const float4* lo, const double4_32a* xyz,
                                            int4 n, Cof<float>& f)
{
  const float4 ha = hi[n.x], hb = hi[n.y], hc = hi[n.z], hd = hi[n.w];
  const float4 la = lo[n.x], lb = lo[n.y], lc = lo[n.z], ld = lo[n.w];
  const float J00 = (hb.x - ha.x) + (lb.x - la.x), J01 = (hc.x - ha.x) + (lc.x - la.x),
              J02 = (hd.x - ha.x) + (ld.x - la.x);
  const float J10 = (hb.y - ha.y) + (lb.y - la.y), J11 = (hc.y - ha.y) + (lc.y - la.y),
              J12 = (hd.y - ha.y) + (ld.y - la.y);
  const float J20 = (hb.z - ha.z) + (lb.z - la.z), J21 = (hc.z - ha.z) + (lc.z - la.z),
              J22 = (hd.z - ha.z) + (ld.z - la.z);
  f.c[0][0] = J11 * J22 - J12 * J21;
  f.c[0][1] = J12 * J20 - J10 * J22;
  f.c[0][2] = J10 * J21 - J11 * J20;
  f.c[1][0] = J02 * J21 - J01 * J22;
  f.c[1][1] = J00 * J22 - J02 * J20;
  f.c[1][2] = J01 * J20 - J00 * J21;
  f.c[2][0] = J01 * J12 - J02 * J11;
  f.c[2][1] = J02 * J10 - J00 * J12;
  f.c[2][2] = J00 * J11 - J01 * J10;
  f.det = J00 * f.c[0][0] + J01 * f.c[0][1] + J02 * f.c[0][2];
  const float n0 = J00 * J00 + J10 * J10 + J20 * J20, n1 = J01 * J01 + J11 * J11 + J21 * J21,
              n2 = J02 * J02 + J12 * J12 + J22 * J22;
  if (fabsf(f.det) * fabsf(f.det) < kFlatTol * kFlatTol * n0 * n1 * n2) {
    Cof<double> g;
    cofactors64(xyz, n, g);
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) f.c[r][k] = (float)g.c[r][k];
    f.det = (float)g.det;
  }
}

template <typename V>
__device__ __forceinline__ void geometry(const AsmArgs& a, int4 n, Cof<V>& f);
template <>
__device__ __forceinline__ void geometry<double>(const AsmArgs& a, int4 n, Cof<double>& f)
{
  cofactors64(a.xyz, n, f);
}
template <>
__device__ __forceinline__ void geometry<float>(const AsmArgs& a, int4 n, Cof<float>& f)
{
  cofactors32(a.xyz_hi, a.xyz_lo, a.xyz, n, f);
}

// P1 stiffness: the 16 entries (k = i*4 + j) of coef * wsum / det * (c_i . c_j).
template <typename V>
__device__ __forceinline__ void p1_stiff(const Cof<V>& f, V s, V* K)
{
  V c[4][3];
  for (int r = 0; r < 3; ++r) {
    c[1][r] = f.c[r][0];
    c[2][r] = f.c[r][1];
    c[3][r] = f.c[r][2];
    c[0][r] = -(c[1][r] + c[2][r] + c[3][r]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i; j < 4; ++j) {
      V v = s * (c[i][0] * c[j][0] + c[i][1] * c[j][1] + c[i][2] * c[j][2]);
      K[i * 4 + j] = v;
      K[j * 4 + i] = v;
    }
}

// The six scaled metric coefficients coef / det * (C_a . C_b), ab = 00,11,22,01,02,12.
template <typename V>
__device__ __forceinline__ void metric(const Cof<V>& f, V s, V g[6])
{
  const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int p = 0; p < 6; ++p)
    g[p] = s * (f.c[0][pa[p]] * f.c[0][pb[p]] + f.c[1][pa[p]] * f.c[1][pb[p]] +
                f.c[2][pa[p]] * f.c[2][pb[p]]);
}

template <int ORDER, typename V>
__global__ void __launch_bounds__(kThreads, 2) k_assemble(AsmArgs a, int stiff)
{
  constexpr int NB = ORDER == 1 ? 4 : 10;
  constexpr int NB2 = NB * NB;
  constexpr int CI = ORDER == 1 ? kChunkP1 : kChunkP2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* acc = reinterpret_cast<V*>(smem_raw);
  V* buf = acc + kAccMax;         // CI * NB2 element-matrix entries + one zero
  V* tab = buf + CI * NB2 + 1;    // 7 * NB2 reference tables
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const BlockDesc d = a.blocks[blockIdx.x];

  for (int i = tid; i < 7 * NB2; i += kThreads) tab[i] = (V)a.tables[i];
  for (int i = tid; i < kAccMax; i += kThreads) acc[i] = V(0);
  if (tid == 0) buf[CI * NB2] = V(0);
  __syncthreads();

  for (int c = 0; c < d.nchunks; ++c) {
    // ---- phase 1: element matrices of this chunk
    if (ORDER == 1) {
      const int it = c * CI + tid;
      if (it < d.item_count) {
        const int e = a.items[d.item_begin + it];
        const int4 n = a.conn[e];
        const V coef = (V)(a.coeff ? a.coeff[e] : a.cconst);
        Cof<V> f;
        geometry<V>(a, n, f);
        V K[16];
        if (stiff) {
          p1_stiff<V>(f, coef * (V)a.wsum / f.det, K);
        } else {
          const V s = coef * f.det;
#pragma unroll
          for (int k = 0; k < 16; ++k) K[k] = s * tab[6 * NB2 + k];
        }
#pragma unroll
        for (int k = 0; k < 16; ++k) buf[k * CI + tid] = K[k];
      }
    } else {
      const int local = tid / kP2ThreadsPerItem, sub = tid % kP2ThreadsPerItem;
      const int it = c * CI + local;
      if (it < d.item_count) {
        const int e = a.items[d.item_begin + it];
        const int4 n = a.conn[e];
        const V coef = (V)(a.coeff ? a.coeff[e] : a.cconst);
        Cof<V> f;
        geometry<V>(a, n, f);
        if (stiff) {
          V g[6];
          metric<V>(f, coef / f.det, g);
          for (int k = sub; k < NB2; k += kP2ThreadsPerItem) {
            V v = g[0] * tab[k];
#pragma unroll
            for (int p = 1; p < 6; ++p) v += g[p] * tab[p * NB2 + k];
            buf[k * CI + local] = v;
          }
        } else {
          const V s = coef * f.det;
          for (int k = sub; k < NB2; k += kP2ThreadsPerItem) buf[k * CI + local] = s * tab[6 * NB2 + k];
        }
      }
    }
    __syncthreads();
    // ---- phase 2: owned-slot reduction
    const int64_t* cp = a.chunk_ptr + (int64_t)(d.chunk_begin + c) * (kWarps + 1);
    const int64_t beg = cp[warp], end = cp[warp + 1];
    for (int64_t o = beg + lane; o < end; o += 32) {
      const uint32_t w = __ldg(a.entries + o);
      acc[(w >> 16) * kThreads + tid] += buf[w & 0xffffu];
    }
    __syncthreads();
  }
  // ---- write the owned rows
  V* out = reinterpret_cast<V*>(a.values);
  for (int r = warp; r < d.row_count; r += kWarps) {
    const int row = a.rows[d.row_begin + r];
    const int base = a.row_acc[d.row_begin + r];
    const int s0 = a.rowptr[row], len = a.rowptr[row + 1] - s0;
    for (int k = lane; k < len; k += 32) out[s0 + k] = acc[base + k];
  }
}

template <int ORDER, typename V>
static size_t assemble_smem()
{
  constexpr int NB2 = ORDER == 1 ? 16 : 100;
  constexpr int CI = ORDER == 1 ? kChunkP1 : kChunkP2;
  return sizeof(V) * (kAccMax + CI * NB2 + 1 + 7 * NB2);
}

template <int ORDER, typename V>
static mg_status launch_assemble_t(const AsmArgs& a, int nblocks, int stiff, cudaStream_t st)
{
  const size_t smem = assemble_smem<ORDER, V>();
  static bool configured = false;
  if (!configured) {
    MG_CUDA(cudaFuncSetAttribute(k_assemble<ORDER, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    configured = true;
  }
  if (nblocks > 0) k_assemble<ORDER, V><<<nblocks, kThreads, smem, st>>>(a, stiff);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

mg_status launch_assemble(mg_plan* p, int op, const double* d_coeff, double c, int quad, int prec,
                          void* d_values, cudaStream_t st)
{
  if (op < MG_OP_STIFF_KAPPA || op > MG_OP_MASS_COEFF)
    return set_error(MG_ERR_INVALID_ARG, "unknown operator " + std::to_string(op));
  if (prec != MG_F64 && prec != MG_F32) return set_error(MG_ERR_INVALID_ARG, "prec must be MG_F64 or MG_F32");
  if (!d_values) return set_error(MG_ERR_INVALID_ARG, "mg_assemble: null values");
  const bool needs_coeff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_MASS_COEFF);
  if (needs_coeff && !d_coeff && p->mesh->n_elem > 0)
    return set_error(MG_ERR_INVALID_ARG, "this operator needs the per-element coefficient array");
  MG_TRY(plan_device(p));
  const RefTables* t = nullptr;
  const double* d_tab = nullptr;
  MG_TRY(plan_tables(p, quad, &t, &d_tab));
  mg_mesh* m = p->mesh;
  AsmArgs a;
  a.blocks = p->d_blocks;
  a.items = p->d_items;
  a.chunk_ptr = p->d_chunk_ptr;
  a.entries = p->d_entries;
  a.rows = p->d_rows;
  a.row_acc = p->d_row_acc;
  a.rowptr = p->d_rowptr;
  a.conn = m->d_conn;
  a.xyz = m->d_xyz;
  a.xyz_hi = m->d_xyz_hi;
  a.xyz_lo = m->d_xyz_lo;
  a.coeff = needs_coeff ? d_coeff : nullptr;
  a.cconst = op == MG_OP_STIFF_CONST ? c : 1.0;
  a.tables = d_tab;
  a.wsum = t->wsum;
  a.values = d_values;
  const int stiff = (op == MG_OP_STIFF_KAPPA || op == MG_OP_STIFF_CONST);
  if (m->order == 1)
    return prec == MG_F64 ? launch_assemble_t<1, double>(a, p->nblocks, stiff, st)
                          : launch_assemble_t<1, float>(a, p->nblocks, stiff, st);
  return prec == MG_F64 ? launch_assemble_t<2, double>(a, p->nblocks, stiff, st)
                        : launch_assemble_t<2, float>(a, p->nblocks, stiff, st);
}

// --------------------------------------------------------------- Dirichlet --
template <typename V>
__global__ void k_dirichlet(int64_t ndof, const int32_t* rowptr, const int32_t* colind,
                            const uint8_t* mask, V* values, double* b)
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
// grad_e = -sum_{i,j} lambda[dof_j] Khat(field i, test j) u[dof_i], Khat the
// kappa = 1 stiffness of element e.
template <int ORDER>
__global__ void k_adjoint(int64_t n_elem, const int4* conn, const int32_t* dofs,
                          const double4_32a* xyz, const double* tables, double wsum,
                          const double* u, const double* lam, double* grad)
{
  constexpr int NB = ORDER == 1 ? 4 : 10, NB2 = NB * NB;
  __shared__ double tab[6 * NB2];
  for (int i = threadIdx.x; i < 6 * NB2; i += blockDim.x) tab[i] = tables[i];
  __syncthreads();
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int4 n = conn[e];
  Cof<double> f;
  cofactors64(xyz, n, f);
  double ue[NB], le[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int dof = dofs[e * NB + i];
    ue[i] = u[dof];
    le[i] = lam[dof];
  }
  double s = 0.0;
  if (ORDER == 1) {
    double K[16];
    p1_stiff<double>(f, wsum / f.det, K);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) s += le[j] * K[i * 4 + j] * ue[i];
  } else {
    double g[6];
    metric<double>(f, 1.0 / f.det, g);
    for (int i = 0; i < NB; ++i) {
      double row = 0.0;
      for (int j = 0; j < NB; ++j) {
        const int k = i * NB + j;
        double v = g[0] * tab[k];
#pragma unroll
        for (int p = 1; p < 6; ++p) v += g[p] * tab[p * NB2 + k];
        row += le[j] * v;
      }
      s += row * ue[i];
    }
  }
  grad[e] = -s;
}

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_assemble(mg_plan* plan, int32_t op, const double* d_coeff, double c, int32_t quad,
                      int32_t prec, void* d_values, void* stream)
{
  if (!plan) return set_error(MG_ERR_INVALID_ARG, "mg_assemble: null plan");
  return launch_assemble(plan, op, d_coeff, c, quad, prec, d_values, (cudaStream_t)stream);
}

mg_status mg_assemble_host(mg_plan* p, int32_t op, const double* h_coeff, double c, int32_t quad,
                           int32_t prec, void* h_values, void* stream)
{
  if (!p || !h_values) return set_error(MG_ERR_INVALID_ARG, "mg_assemble_host: null argument");
  MG_TRY(plan_device(p));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t vbytes = (size_t)p->nnz * (prec == MG_F64 ? 8 : 4);
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
  MG_CUDA(cudaMemcpyAsync(h_values, p->d_tmp_values, vbytes, cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  return MG_OK;
}

mg_status mg_apply_dirichlet(mg_plan* p, const uint8_t* d_mask, int32_t prec, void* d_values,
                             double* d_b, void* stream)
{
  if (!p || !d_mask || !d_values) return set_error(MG_ERR_INVALID_ARG, "mg_apply_dirichlet: null argument");
  if (prec != MG_F64 && prec != MG_F32) return set_error(MG_ERR_INVALID_ARG, "bad precision");
  MG_TRY(plan_device(p));
  const int threads = 256;
  const int blocks = (int)((p->ndof + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (blocks > 0) {
    if (prec == MG_F64)
      k_dirichlet<double><<<blocks, threads, 0, st>>>(p->ndof, p->d_rowptr, p->d_colind, d_mask,
                                                      (double*)d_values, d_b);
    else
      k_dirichlet<float><<<blocks, threads, 0, st>>>(p->ndof, p->d_rowptr, p->d_colind, d_mask,
                                                     (float*)d_values, d_b);
  }
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

mg_status mg_adjoint_grad(mg_plan* p, const double* d_u, const double* d_lambda, int32_t quad,
                          double* d_grad, void* stream)
{
  if (!p || !d_u || !d_lambda || !d_grad) return set_error(MG_ERR_INVALID_ARG, "mg_adjoint_grad: null argument");
  MG_TRY(plan_device(p));
  const RefTables* t = nullptr;
  const double* d_tab = nullptr;
  MG_TRY(plan_tables(p, quad, &t, &d_tab));
  mg_mesh* m = p->mesh;
  const int threads = 256;
  const int blocks = (int)((m->n_elem + threads - 1) / threads);
  cudaStream_t st = (cudaStream_t)stream;
  if (blocks > 0) {
    if (m->order == 1)
      k_adjoint<1><<<blocks, threads, 0, st>>>(m->n_elem, m->d_conn, m->d_dofs, m->d_xyz, d_tab,
                                               t->wsum, d_u, d_lambda, d_grad);
    else
      k_adjoint<2><<<blocks, threads, 0, st>>>(m->n_elem, m->d_conn, m->d_dofs, m->d_xyz, d_tab,
                                               t->wsum, d_u, d_lambda, d_grad);
  }
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

mg_status mg_assemble_rhs(mg_plan* p, const double* d_field, const double* d_elem_scale, int32_t quad,
                          double* d_b, void* stream)
{
  if (!p || !d_b) return set_error(MG_ERR_INVALID_ARG, "mg_assemble_rhs: null argument");
  MG_TRY(plan_device(p));
  cudaStream_t st = (cudaStream_t)stream;
  // b = M_s f with M_s the (element-scaled) mass matrix: the same integral as
  // sum_e s_e int_e f_h phi_i, since f_h = sum_k f_k phi_k on every element.
  const size_t vbytes = (size_t)p->nnz * 8;
  if (p->tmp_values_bytes < vbytes) {
    cudaFree(p->d_tmp_values);
    p->d_tmp_values = nullptr;
    p->tmp_values_bytes = 0;
    MG_CUDA(cudaMalloc(&p->d_tmp_values, vbytes));
    p->tmp_values_bytes = vbytes;
  }
  MG_TRY(launch_assemble(p, d_elem_scale ? MG_OP_MASS_COEFF : MG_OP_MASS, d_elem_scale, 1.0, quad, MG_F64,
                         p->d_tmp_values, st));
  if (d_field) return launch_spmv(p, MG_F64, p->d_tmp_values, d_field, d_b, st);
  return launch_rowsum(p, (const double*)p->d_tmp_values, d_b, st);
}

}  // extern "C"
