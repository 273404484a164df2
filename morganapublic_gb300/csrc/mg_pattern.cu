// Mesh preprocessing on the GPU: edge enumeration / numbering and the CSR
// pattern, each giving the host build's arrays bit for bit.
//
// Edges (connect3d.hpp:417-491 with pMapItem / pMapItemShare numbering in
// morganaPublic): the 6 E element-edge incidences as keys min << 32 | max,
// radix-sorted with the incidence index as value (a stable sort, so the first
// incidence of an edge heads its run); run heads give the lexicographic edge
// ids (the LEX rule), and a second sort of the edges by first incidence gives
// the FIRST rule's ids.
//
// CSR pattern on the GPU: the same rows and columns as the host build (the
// union of every element's (test dof, field dof) couplings, columns sorted,
// explicit zeros kept -- traitsMatrixBuilder.hpp:443-544 and the insert /
// GlobalAssemble of buildEpetraCrs, :363-441, in morganaPublic), computed as
//   1. one 64-bit key row << 32 | col per element coupling (E nb^2 keys),
//   2. a radix sort of the keys and removal of duplicates (CUB),
//   3. row starts by binary search over the sorted unique keys.
// The pattern is copied to the host (the export calls and the boundary-multiplier
// build read it there) and, for the device plan build, kept on the device.
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

// local edge j of a tet joins its vertices kEdge[j][0] and kEdge[j][1]
__constant__ int kEdgeDev[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

__global__ void __launch_bounds__(256) k_edge_keys(int64_t M, const int32_t* __restrict__ conn,
                                                   unsigned long long* __restrict__ keys, int32_t* __restrict__ vals)
{
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= M) return;
  const int64_t e = t / 6;
  const int j = (int)(t % 6);
  const uint32_t a = (uint32_t)conn[4 * e + kEdgeDev[j][0]], b = (uint32_t)conn[4 * e + kEdgeDev[j][1]];
  keys[t] = ((unsigned long long)min(a, b) << 32) | max(a, b);
  vals[t] = (int32_t)t;
}

__global__ void __launch_bounds__(256) k_edge_heads(int64_t M, const unsigned long long* __restrict__ keys,
                                                    int32_t* __restrict__ head)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < M) head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

// first incidence of each edge (lexicographic id g = lex[k] - 1 at its run head)
__global__ void __launch_bounds__(256) k_edge_first(int64_t M, const int32_t* __restrict__ head,
                                                    const int32_t* __restrict__ lex, const int32_t* __restrict__ inc,
                                                    int32_t* __restrict__ first, int32_t* __restrict__ ids)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < M && head[k]) {
    first[lex[k] - 1] = inc[k];
    ids[lex[k] - 1] = lex[k] - 1;
  }
}

// gid_of_lex from the edges sorted by first incidence (FIRST rule)
__global__ void __launch_bounds__(256) k_edge_rank(int64_t nE, const int32_t* __restrict__ sorted_g,
                                                   int32_t* __restrict__ gid_of_lex)
{
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < nE) gid_of_lex[sorted_g[r]] = (int32_t)r;
}

__global__ void __launch_bounds__(256) k_edge_scatter(int64_t M, const int32_t* __restrict__ lex,
                                                      const int32_t* __restrict__ inc,
                                                      const int32_t* __restrict__ gid_of_lex,
                                                      int32_t* __restrict__ elem_edge)
{
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < M) elem_edge[inc[k]] = gid_of_lex ? gid_of_lex[lex[k] - 1] : lex[k] - 1;
}

// end points of each edge, oriented as in its first incidence
__global__ void __launch_bounds__(256) k_edge_nodes(int64_t nE, const int32_t* __restrict__ first,
                                                    const int32_t* __restrict__ gid_of_lex,
                                                    const int32_t* __restrict__ conn, int32_t* __restrict__ nodes)
{
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nE) return;
  const int64_t t = first[g], e = t / 6;
  const int j = (int)(t % 6);
  const int64_t gid = gid_of_lex ? gid_of_lex[g] : g;
  nodes[2 * gid] = conn[4 * e + kEdgeDev[j][0]];
  nodes[2 * gid + 1] = conn[4 * e + kEdgeDev[j][1]];
}

static int key_bits(int64_t n)  // bits that hold every value < n
{
  int b = 0;
  while (b < 62 && (1ll << b) < n) ++b;
  return b;
}

struct EdgeBuffers {
  int32_t *conn = nullptr, *vals = nullptr, *vals_s = nullptr, *head = nullptr, *lex = nullptr, *first = nullptr,
          *ids = nullptr, *ids_s = nullptr, *first_s = nullptr, *gid = nullptr, *elem_edge = nullptr,
          *nodes = nullptr;
  unsigned long long *keys = nullptr, *keys_s = nullptr;
  void* tmp = nullptr;
  ~EdgeBuffers()
  {
    for (void* q : {(void*)conn, (void*)vals, (void*)vals_s, (void*)head, (void*)lex, (void*)first, (void*)ids,
                    (void*)ids_s, (void*)first_s, (void*)gid, (void*)elem_edge, (void*)nodes, (void*)keys,
                    (void*)keys_s, tmp})
      cudaFree(q);
  }
};

mg_status build_edges_device(mg_mesh* m, cudaStream_t st)
{
  if (m->n_edges >= 0) return MG_OK;
  const int64_t N = m->n_nodes, E = m->n_elem, M = 6 * E;
  if (M >= INT32_MAX) return set_error(MG_ERR_SIZE, "device edge build: more than 2^31 edge incidences");
  if (M == 0) {
    m->elem_edge.clear();
    m->edge_nodes.clear();
    m->n_edges = 0;
    return MG_OK;
  }
  EdgeBuffers d;
  const size_t i4 = sizeof(int32_t) * M, k8 = sizeof(unsigned long long) * M;
  MG_CUDA(cudaMalloc(&d.conn, sizeof(int32_t) * 4 * E));
  for (int32_t** q : {&d.vals, &d.vals_s, &d.head, &d.lex, &d.first, &d.ids, &d.ids_s, &d.first_s, &d.gid,
                      &d.elem_edge})
    MG_CUDA(cudaMalloc(q, i4));
  MG_CUDA(cudaMalloc(&d.keys, k8));
  MG_CUDA(cudaMalloc(&d.keys_s, k8));
  size_t b1 = 0, b2 = 0, b3 = 0;
  const int kb = 32 + key_bits(N), fb = key_bits(M);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, b1, d.keys, d.keys_s, d.vals, d.vals_s, (int)M, 0, kb, st));
  MG_CUDA(cub::DeviceScan::InclusiveSum(nullptr, b2, d.head, d.lex, (int)M, st));
  MG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, b3, d.first, d.first_s, d.ids, d.ids_s, (int)M, 0, fb, st));
  MG_CUDA(cudaMalloc(&d.tmp, std::max({b1, b2, b3})));
  MG_CUDA(cudaMemcpyAsync(d.conn, m->conn.data(), sizeof(int32_t) * 4 * E, cudaMemcpyHostToDevice, st));
  const int T = 256;
  const int gm = (int)((M + T - 1) / T);
  k_edge_keys<<<gm, T, 0, st>>>(M, d.conn, d.keys, d.vals);
  MG_CUDA(cub::DeviceRadixSort::SortPairs(d.tmp, b1, d.keys, d.keys_s, d.vals, d.vals_s, (int)M, 0, kb, st));
  k_edge_heads<<<gm, T, 0, st>>>(M, d.keys_s, d.head);
  MG_CUDA(cub::DeviceScan::InclusiveSum(d.tmp, b2, d.head, d.lex, (int)M, st));
  int32_t nE = 0;
  MG_CUDA(cudaMemcpyAsync(&nE, d.lex + (M - 1), sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  k_edge_first<<<gm, T, 0, st>>>(M, d.head, d.lex, d.vals_s, d.first, d.ids);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaStreamSynchronize(st));
  const int ge = (int)((nE + T - 1) / T);
  const int32_t* gid = nullptr;
  if (m->edge_rule == MG_EDGES_FIRST) {
    // edges ordered by their first incidence (distinct values)
    MG_CUDA(cub::DeviceRadixSort::SortPairs(d.tmp, b3, d.first, d.first_s, d.ids, d.ids_s, (int)nE, 0, fb, st));
    k_edge_rank<<<ge, T, 0, st>>>(nE, d.ids_s, d.gid);
    gid = d.gid;
  }
  k_edge_scatter<<<gm, T, 0, st>>>(M, d.lex, d.vals_s, gid, d.elem_edge);
  MG_CUDA(cudaMalloc(&d.nodes, sizeof(int32_t) * 2 * std::max<int64_t>(nE, 1)));
  k_edge_nodes<<<ge, T, 0, st>>>(nE, d.first, gid, d.conn, d.nodes);
  MG_CUDA(cudaGetLastError());
  m->elem_edge.resize(M);
  m->edge_nodes.resize(2 * (int64_t)nE);
  MG_CUDA(cudaMemcpyAsync(m->elem_edge.data(), d.elem_edge, i4, cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaMemcpyAsync(m->edge_nodes.data(), d.nodes, sizeof(int32_t) * 2 * nE, cudaMemcpyDeviceToHost, st));
  MG_CUDA(cudaStreamSynchronize(st));
  m->n_edges = nE;
  return MG_OK;
}

mg_status build_pattern_device(mg_plan* p, cudaStream_t st, bool keep_device)
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
  if (n == 0) {  // no elements: every row empty
    if (keep_device) {
      MG_CUDA(cudaMalloc(&p->d_rowptr, sizeof(int32_t) * (nd + 1)));
      MG_CUDA(cudaMalloc(&p->d_colind, sizeof(int32_t)));
      MG_CUDA(cudaMemsetAsync(p->d_rowptr, 0, sizeof(int32_t) * (nd + 1), st));
      MG_CUDA(cudaStreamSynchronize(st));
    }
    return MG_OK;
  }
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
  if (nnz >= INT32_MAX) return set_error(MG_ERR_SIZE, "nnz above 2^31-1");
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
  if (keep_device) {  // the device copies become the plan's (the plan's device state is built from them)
    p->d_rowptr = d.rowptr;
    p->d_colind = d.colind;
    d.rowptr = nullptr;
    d.colind = nullptr;
  }
  return MG_OK;
}

}  // namespace mg
