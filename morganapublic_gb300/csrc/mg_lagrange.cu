// Boundary multipliers on the GPU: values of B = opLA3dA, of the saddle matrix
// [K B^T; B 0], and the products with them.
//
// B is assembled in two deterministic passes:
//   k_face_matrix  one thread per boundary face: its nt x nb local matrix
//                  (mg_lagrange.cuh) into a staging array, face-major;
//   k_gather_sum   one thread per entry of B: the staged values it sums, in the
//                  reference's insertion order (element, local face, face
//                  vertex, basis), from the host-built list of the entry.
// No atomics, so every run gives the same bits.  The work is O(boundary faces)
// (n^2 against the volume operator's n^3) and runs in native FP64.
// The saddle values are a gather from K's and B's values through a per-entry
// source map (plus, for setMTM / setMMT, one thread per entry of B^T B or
// B B^T summing its products); the products with the matrices use the CSR SpMV
// kernel of mg_solve.cu.
#include <algorithm>
#include <climits>

#include "mg_internal.h"
#include "mg_lagrange.cuh"

namespace mg {

namespace {

constexpr int kFaceThreads = 256;

int grid_for(int64_t n)
{
  const int64_t b = (n + kFaceThreads - 1) / kFaceThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 65535));
}

template <int NB, int NT>
__global__ void __launch_bounds__(kFaceThreads) k_face_matrix(int64_t n_faces, const int2* __restrict__ faces,
                                                          const int4* __restrict__ conn,
                                                          const double4_32a* __restrict__ xyz, FaceRule rule,
                                                          double* __restrict__ out)
{
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < n_faces; f += (int64_t)gridDim.x * blockDim.x) {
    const int2 fe = faces[f];
    const int4 c = conn[fe.x];
    const int v[4] = {c.x, c.y, c.z, c.w};
    double P[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double4_32a p = xyz[v[face_vertex(fe.y, a)]];
      P[a][0] = p.x;
      P[a][1] = p.y;
      P[a][2] = p.z;
    }
    double mat[NT * NB];
    face_matrix<NB, NT>(P, fe.y, rule, mat);
    double* o = out + f * (NT * NB);
#pragma unroll
    for (int k = 0; k < NT * NB; ++k) o[k] = mat[k];
  }
}

// vals[k] = sum of src_vals[src[j]] over j in [ptr[k], ptr[k+1]), in list order
__global__ void __launch_bounds__(kFaceThreads) k_gather_sum(int64_t n, const int32_t* __restrict__ ptr,
                                                         const int32_t* __restrict__ src,
                                                         const double* __restrict__ src_vals,
                                                         double* __restrict__ vals)
{
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    const int32_t j1 = ptr[k + 1];
    for (int32_t j = ptr[k]; j < j1; ++j) s += src_vals[src[j]];
    vals[k] = s;
  }
}

// Saddle entry k: K's entry src (>= 0), B's entry -(src + 1), eye_lam
// (kSrcLamDiag) or zero (kSrcZero, a B^T B entry outside K)
__global__ void __launch_bounds__(kFaceThreads) k_saddle_fill(int64_t n, const int32_t* __restrict__ src,
                                                          const double* __restrict__ kv,
                                                          const double* __restrict__ bv, double eye_lam,
                                                          double* __restrict__ out)
{
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = src[k];
    out[k] = s >= 0 ? kv[s] : (s == kSrcLamDiag ? eye_lam : (s == kSrcZero ? 0.0 : bv[-(s + 1)]));
  }
}

// Product entry m (B^T B or B B^T): scale * sum of bv[k1] bv[k2] over its
// pairs (in their fixed order), added to its saddle entry (one entry per m: no
// atomics)
__global__ void __launch_bounds__(kFaceThreads) k_saddle_products(int64_t n, const int32_t* __restrict__ pair_ptr,
                                                         const int2* __restrict__ pairs,
                                                         const int32_t* __restrict__ slot,
                                                         const double* __restrict__ bv, double scale,
                                                         double* __restrict__ out)
{
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < n; m += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    const int32_t j1 = pair_ptr[m + 1];
    for (int32_t j = pair_ptr[m]; j < j1; ++j) {
      const int2 pr = pairs[j];
      s += bv[pr.x] * bv[pr.y];
    }
    out[slot[m]] += scale * s;
  }
}

// Adds eye to the diagonal of the field block, at each row's diagonal entry
// (s_diag[r]; rows without one, dofs outside every element, are left alone).
__global__ void __launch_bounds__(kFaceThreads) k_saddle_eye(int64_t nd, const int32_t* __restrict__ s_diag,
                                                         double eye, double* __restrict__ out)
{
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nd; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = s_diag[r];
    if (d >= 0) out[d] += eye;
  }
}

}  // namespace

}  // namespace mg

using namespace mg;

extern "C" {

mg_status mg_lagrange_assemble(mg_lagrange* lg, int32_t quad, double* d_b_values, void* stream)
{
  NvtxRange nvtx_range("mg_lagrange_assemble");
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble: null handle");
  FaceRule rule{};
  if (!face_rule(quad, &rule)) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble: face card must be 1, 3, 4 or 6");
  if (lg->nnz_b == 0) return MG_OK;
  if (!d_b_values) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble: null values");
  MG_TRY(lagrange_device(lg));
  cudaStream_t st = (cudaStream_t)stream;
  const mg_mesh* m = lg->plan->mesh;
  const int g = grid_for(lg->n_faces);
  const int64_t F = lg->n_faces;
#define MG_FACE_LAUNCH(NB_, NT_) \
  k_face_matrix<NB_, NT_><<<g, kFaceThreads, 0, st>>>(F, lg->d_faces, m->d_conn, m->d_xyz, rule, lg->d_face_mat)
  if (lg->nb == 4) {
    if (lg->nt == 3) MG_FACE_LAUNCH(4, 3);
    else if (lg->nt == 1) MG_FACE_LAUNCH(4, 1);
    else MG_FACE_LAUNCH(4, 6);
  } else {
    if (lg->nt == 3) MG_FACE_LAUNCH(10, 3);
    else if (lg->nt == 1) MG_FACE_LAUNCH(10, 1);
    else MG_FACE_LAUNCH(10, 6);
  }
#undef MG_FACE_LAUNCH
  MG_CUDA(cudaGetLastError());
  k_gather_sum<<<grid_for(lg->nnz_b), kFaceThreads, 0, st>>>(lg->nnz_b, lg->d_b_src_ptr, lg->d_b_src, lg->d_face_mat,
                                                          d_b_values);
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

mg_status mg_lagrange_assemble_host(mg_lagrange* lg, int32_t quad, double* h_b_values)
{
  NvtxRange nvtx_range("mg_lagrange_assemble_host");
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble_host: null handle");
  FaceRule rule{};
  if (!face_rule(quad, &rule))
    return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble_host: face card must be 1, 3, 4 or 6");
  if (lg->nnz_b == 0) return MG_OK;
  if (!h_b_values) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_assemble_host: null values");
  double* d = nullptr;
  MG_CUDA(cudaMalloc(&d, sizeof(double) * lg->nnz_b));
  mg_status s = mg_lagrange_assemble(lg, quad, d, nullptr);
  if (s == MG_OK) {
    const cudaError_t e = cudaMemcpy(h_b_values, d, sizeof(double) * lg->nnz_b, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_error(e, "cudaMemcpy(B values)");
  }
  cudaFree(d);
  return s;
}

mg_status mg_saddle_assemble(mg_lagrange* lg, const double* d_k_values, const double* d_b_values,
                             const mg_saddle_scales* scales, double* d_values, void* stream)
{
  NvtxRange nvtx_range("mg_saddle_assemble");
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_saddle_assemble: null handle");
  const mg_saddle_scales sc = scales ? *scales : mg_saddle_scales{0.0, 0.0, 0.0, 0.0};
  const double eye_field = sc.eye_field, eye_lam = sc.eye_lam, mtm_scale = sc.mtm, mmt_scale = sc.mmt;
  if (eye_lam != 0.0 && !lg->lam_diag)
    return set_error(MG_ERR_INVALID_ARG, "mg_saddle_assemble: eye_lam needs a pattern built with MG_SADDLE_LAM_DIAG");
  if (mtm_scale != 0.0 && !lg->mtm)
    return set_error(MG_ERR_INVALID_ARG, "mg_saddle_assemble: mtm needs a pattern built with MG_SADDLE_MTM");
  if (mmt_scale != 0.0 && !lg->mmt)
    return set_error(MG_ERR_INVALID_ARG, "mg_saddle_assemble: mmt needs a pattern built with MG_SADDLE_MMT");
  if (lg->nnz_s == 0) return MG_OK;
  if (!d_values || (lg->plan->nnz && !d_k_values) || (lg->nnz_b && !d_b_values))
    return set_error(MG_ERR_INVALID_ARG, "mg_saddle_assemble: null argument");
  MG_TRY(lagrange_device(lg));
  cudaStream_t st = (cudaStream_t)stream;
  k_saddle_fill<<<grid_for(lg->nnz_s), kFaceThreads, 0, st>>>(lg->nnz_s, lg->d_s_src, d_k_values, d_b_values, eye_lam,
                                                           d_values);
  MG_CUDA(cudaGetLastError());
  if (eye_field != 0.0 && lg->ndof > 0) {
    k_saddle_eye<<<grid_for(lg->ndof), kFaceThreads, 0, st>>>(lg->ndof, lg->d_s_diag, eye_field, d_values);
    MG_CUDA(cudaGetLastError());
  }
  if (mtm_scale != 0.0 && lg->nnz_m > 0) {
    k_saddle_products<<<grid_for(lg->nnz_m), kFaceThreads, 0, st>>>(lg->nnz_m, lg->d_m_pair_ptr, lg->d_m_pairs,
                                                                    lg->d_m_slot, d_b_values, mtm_scale, d_values);
    MG_CUDA(cudaGetLastError());
  }
  if (mmt_scale != 0.0 && lg->nnz_p > 0) {
    k_saddle_products<<<grid_for(lg->nnz_p), kFaceThreads, 0, st>>>(lg->nnz_p, lg->d_p_pair_ptr, lg->d_p_pairs,
                                                                    lg->d_p_slot, d_b_values, mmt_scale, d_values);
    MG_CUDA(cudaGetLastError());
  }
  return MG_OK;
}

mg_status mg_saddle_spmv(mg_lagrange* lg, const double* d_values, const double* d_x, double* d_y, void* stream)
{
  NvtxRange nvtx_range("mg_saddle_spmv");
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_saddle_spmv: null handle");
  const int64_t rows = lg->ndof + lg->nl;
  if (rows == 0) return MG_OK;
  if (!d_values || !d_x || !d_y) return set_error(MG_ERR_INVALID_ARG, "mg_saddle_spmv: null argument");
  MG_TRY(lagrange_device(lg));
  return launch_spmv_csr(rows, lg->nnz_s, lg->d_s_rowptr, lg->d_s_colind, d_values, d_x, d_y, (cudaStream_t)stream);
}

mg_status mg_lagrange_apply(mg_lagrange* lg, const double* d_b_values, const double* d_u, double* d_g, void* stream)
{
  NvtxRange nvtx_range("mg_lagrange_apply");
  if (!lg) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_apply: null handle");
  if (lg->nl == 0) return MG_OK;
  if (!d_b_values || !d_u || !d_g) return set_error(MG_ERR_INVALID_ARG, "mg_lagrange_apply: null argument");
  MG_TRY(lagrange_device(lg));
  return launch_spmv_csr(lg->nl, lg->nnz_b, lg->d_b_rowptr, lg->d_b_colind, d_b_values, d_u, d_g,
                         (cudaStream_t)stream);
}

}  // extern "C"
