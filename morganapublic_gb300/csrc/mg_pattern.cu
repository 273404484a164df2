// CSR pattern on the GPU: the same rows and columns as the host build (the
// union of every element's (test dof, field dof) couplings, columns sorted,
// explicit zeros kept -- traitsMatrixBuilder.hpp:443-544 and the insert /
// GlobalAssemble of buildEpetraCrs, :363-441, in morganaPublic), computed as
//   1. one 64-bit key row << 32 | col per element coupling (E nb^2 keys),
//   2. a radix sort of the keys and removal of duplicates (CUB),
//   3. row starts by binary search over the sorted unique keys.
// The assembly schedule is then built on the host from the downloaded pattern.
#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "mg_internal.h"

namespace mg {

// one thread per (element, test basis j): the element's nb couplings of row dofs[j]
__global__ void __launch_bounds__(256) k_pattern_keys(int64_t n_elem, int nb, const int32_t* __restrict__ dofs,
                                                      unsigned long long* __restrict__ keys)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n_elem * nb) return;
  const int64_t e = t / nb;
  const unsigned long long row = (unsigned long long)(uint32_t)dofs[t];
  unsigned long long* out = keys + t * nb;
  for (int i = 0; i < nb; ++i) out[i] = (row << 32) | (uint32_t)dofs[e * nb + i];
}

// rowptr[r] = the first unique key with row >= r; colind from the low halves
__global__ void __launch_bounds__(256) k_pattern_rows(int64_t nd, int64_t nnz, const unsigned long long* __restrict__ keys,
                                                      int32_t* __restrict__ rowptr)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r > nd) return;
  const unsigned long long target = (unsigned long long)r << 32;
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < target) lo = mid + 1;
    else hi = mid;
  }
  rowptr[r] = (int32_t)lo;
}

__global__ void __launch_bounds__(256) k_pattern_cols(int64_t nnz, const unsigned long long* __restrict__ keys,
                                                      int32_t* __restrict__ colind)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < nnz) colind[k] = (int32_t)(uint32_t)keys[k];
}

// Device buffers of one build, freed on every exit path.
struct PatternBuffers {
  unsigned long long *a = nullptr, *b = nullptr;
  void* tmp = nullptr;
  int64_t* count = nullptr;
  int32_t *rowptr = nullptr, *colind = nullptr;
  ~PatternBuffers()
  {
    cudaFree(a);
    cudaFree(b);
    cudaFree(tmp);
    cudaFree(count);
    cudaFree(rowptr);
    cudaFree(colind);
  }
};

mg_status build_pattern_device(mg_plan* p, cudaStream_t st)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = m->ndof, n = E * nb * nb;
  if (n >= INT32_MAX) return set_error(MG_ERR_SIZE, "device pattern build: more than 2^31 element couplings");
  if (nd >= INT32_MAX) return set_error(MG_ERR_SIZE, "device pattern build: ndof above 2^31");
  MG_TRY(mesh_device(m));
  p->ndof = nd;
  p->rowptr.assign(nd + 1, 0);
  p->colind.clear();
  p->nnz = 0;
  if (n == 0) return MG_OK;
  PatternBuffers d;
  MG_CUDA(cudaMalloc(&d.a, sizeof(unsigned long long) * n));
  MG_CUDA(cudaMalloc(&d.b, sizeof(unsigned long long) * n));
  MG_CUDA(cudaMalloc(&d.count, sizeof(int64_t)));
  int end_bit = 32;
  while (end_bit < 64 && (1ll << (end_bit - 32)) < nd) ++end_bit;  // rows < nd
  size_t sort_bytes = 0, uniq_bytes = 0;
  MG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, d.a, d.b, (int)n, 0, end_bit, st));
  MG_CUDA(cub::DeviceSelect::Unique(nullptr, uniq_bytes, d.b, d.a, d.count, (int)n, st));
  MG_CUDA(cudaMalloc(&d.tmp, std::max(sort_bytes, uniq_bytes)));
  const int threads = 256;
  k_pattern_keys<<<(int)((E * nb + threads - 1) / threads), threads, 0, st>>>(E, nb, m->d_dofs, d.a);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cub::DeviceRadixSort::SortKeys(d.tmp, sort_bytes, d.a, d.b, (int)n, 0, end_bit, st));
  MG_CUDA(cub::DeviceSelect::Unique(d.tmp, uniq_bytes, d.b, d.a, d.count, (int)n, st));
  int64_t nnz = 0;
  MG_CUDA(cudaMemcpyAsync(&nnz, d.count, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  MG_CUDA(cudaMalloc(&d.rowptr, sizeof(int32_t) * (nd + 1)));
  MG_CUDA(cudaMalloc(&d.colind, sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
  k_pattern_rows<<<(int)((nd + 1 + threads - 1) / threads), threads, 0, st>>>(nd, nnz, d.a, d.rowptr);
  k_pattern_cols<<<(int)((nnz + threads - 1) / threads), threads, 0, st>>>(nnz, d.a, d.colind);
  MG_CUDA(cudaGetLastError());
  p->colind.resize(nnz);
  MG_CUDA(cudaMemcpyAsync(p->rowptr.data(), d.rowptr, sizeof(int32_t) * (nd + 1), cudaMemcpyDeviceToHost, st));
  if (nnz > 0)
    MG_CUDA(cudaMemcpyAsync(p->colind.data(), d.colind, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  p->nnz = nnz;
  for (int64_t r = 0; r < nd; ++r)
    if (p->rowptr[r + 1] - p->rowptr[r] > kAccMax) return set_error(MG_ERR_SIZE, "a CSR row has more than 8192 entries");
  return MG_OK;
}

}  // namespace mg
