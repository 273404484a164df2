// CSR pattern and GPU assembly schedule (host side).
//
// Pattern: the union of element couplings with sorted columns and explicit
// zeros kept -- the matrix traitsMatrixBuilder::buildEpetraCrs leaves behind
// after Epetra_FECrsMatrix::GlobalAssemble
// (src/morganaFiniteElements/traitsMatrixBuilder.hpp:363-544 in morganaPublic).
//
// Schedule: the rows (dofs) are cut into blocks along a Morton curve of the dof
// positions, each holding at most kAccMax CSR entries.  One CTA owns one block:
// it recomputes every element touching one of its rows ("items", ordered along
// a Morton curve of the element centroids) and sums each owned CSR entry in
// shared memory.  The items are
// processed in chunks; the contributions of a chunk are sorted by accumulator
// slot into segments (one per slot, in element order), and the segments are
// dealt to the CTA's threads longest-first to the least-loaded thread.  A
// thread sums each of its segments sequentially and adds the sum to the slot,
// so within a chunk every slot is written by exactly one thread: no atomics, no
// second pass, and a summation order fixed by the plan (bitwise reproducible).
// Each thread's words are interleaved by lane ([k][lane]) within its warp and
// padded to the warp's longest list, so the chunk is one contiguous, 128-byte
// aligned region the kernel stages into shared memory with a bulk copy.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

#include <omp.h>
#include <parallel/algorithm>

#include "mg_internal.h"

namespace mg {

static uint64_t spread21(uint64_t v)
{
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

static mg_status build_pattern(mg_plan* p)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = m->ndof;
  // dof -> incident elements (the order inside a row does not matter: the
  // row's columns are de-duplicated and sorted below)
  std::vector<int64_t> start(nd + 1, 0);
#pragma omp parallel for
  for (int64_t k = 0; k < E * nb; ++k) {
#pragma omp atomic
    start[m->dofs[k] + 1]++;
  }
  for (int64_t r = 0; r < nd; ++r) start[r + 1] += start[r];
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  std::vector<int32_t> inc(E * nb);
#pragma omp parallel for
  for (int64_t k = 0; k < E * nb; ++k) {
    int64_t slot;
#pragma omp atomic capture
    slot = fill[m->dofs[k]]++;
    inc[slot] = (int32_t)(k / nb);
  }
  // one pass over the rows: the union of the incident elements' dofs,
  // de-duplicated with a per-thread stamp array (so only the ~15 unique columns
  // of a P1 row are sorted), kept per thread and copied after the prefix sum
  std::vector<int32_t> len(nd, 0);
  int bad = 0;
  const int nth = std::max(1, omp_get_max_threads());
  std::vector<std::vector<int32_t>> cols(nth);
  std::vector<int64_t> chunk_row0(nth + 1, 0);
#pragma omp parallel num_threads(nth)
  {
    const int t = omp_get_thread_num();
    const int64_t r0 = nd * t / nth, r1 = nd * (t + 1) / nth;
    chunk_row0[t] = r0;
    std::vector<int32_t> stamp(nd, -1);
    std::vector<int32_t>& out = cols[t];
    std::vector<int32_t> tmp;
    for (int64_t r = r0; r < r1; ++r) {
      tmp.clear();
      for (int64_t k = start[r]; k < start[r + 1]; ++k)
        for (int i = 0; i < nb; ++i) {
          const int32_t c = m->dofs[(int64_t)inc[k] * nb + i];
          if (stamp[c] != (int32_t)r) {
            stamp[c] = (int32_t)r;
            tmp.push_back(c);
          }
        }
      std::sort(tmp.begin(), tmp.end());
      len[r] = (int32_t)tmp.size();
      if (len[r] > kAccMax) bad = 1;
      out.insert(out.end(), tmp.begin(), tmp.end());
    }
  }
  if (bad) return set_error(MG_ERR_SIZE, "a CSR row has more than 8192 entries");
  p->rowptr.assign(nd + 1, 0);
  for (int64_t r = 0; r < nd; ++r) {
    int64_t next = (int64_t)p->rowptr[r] + len[r];
    if (next >= INT32_MAX) return set_error(MG_ERR_SIZE, "nnz above 2^31-1");
    p->rowptr[r + 1] = (int32_t)next;
  }
  p->nnz = p->rowptr[nd];
  p->colind.resize(p->nnz);
#pragma omp parallel for num_threads(nth)
  for (int t = 0; t < nth; ++t)
    std::copy(cols[t].begin(), cols[t].end(), p->colind.begin() + p->rowptr[chunk_row0[t]]);
  p->ndof = nd;
  return MG_OK;
}

// SMs of the current device (one persistent assembly CTA each); GB300's 152
// when no device is visible.
static int64_t sm_count_hint()
{
  int n = 0, dev = 0, sms = 0;
  if (cudaGetDeviceCount(&n) == cudaSuccess && n > 0 && cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
    return sms;
  cudaGetLastError();
  return 152;
}

// Block count of the schedule: the smallest nbk with W / nbk + wmax <= kAccMax
// (W the total row weight, wmax the largest), raised to a multiple of `sms` when
// it is above half of it.
int64_t schedule_block_count(int64_t wtot, int64_t wmax, int64_t sms)
{
  if (wtot <= 0) return 1;
  const int64_t room = std::max<int64_t>(1, kAccMax - wmax);
  int64_t nbk = std::max<int64_t>(1, (wtot + room - 1) / room);
  if (nbk > sms / 2) nbk = (nbk + sms - 1) / sms * sms;
  return nbk;
}

static mg_status build_schedule(mg_plan* p, HostSchedule* hs)
{
  mg_mesh* m = p->mesh;
  const int nb = m->nb, nb2 = nb * nb, CI = chunk_items(m->order);
  const int64_t E = m->n_elem, nd = p->ndof, N = m->n_nodes;
  if (CI * nb2 + 1 > 0xffff) return set_error(MG_ERR_SIZE, "chunk buffer above 16-bit index");
  // dof positions and Morton keys
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < N; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], m->xyz[3 * i + k]);
      hi[k] = std::max(hi[k], m->xyz[3 * i + k]);
    }
  std::vector<uint64_t> key(nd);
#pragma omp parallel for
  for (int64_t d = 0; d < nd; ++d) {
    double x[3];
    if (d < N) {
      for (int k = 0; k < 3; ++k) x[k] = m->xyz[3 * d + k];
    } else {
      const int32_t a = m->edge_nodes[2 * (d - N)], b = m->edge_nodes[2 * (d - N) + 1];
      for (int k = 0; k < 3; ++k) x[k] = 0.5 * (m->xyz[3 * (int64_t)a + k] + m->xyz[3 * (int64_t)b + k]);
    }
    uint64_t c = 0;
    for (int k = 0; k < 3; ++k) {
      double t = hi[k] > lo[k] ? (x[k] - lo[k]) / (hi[k] - lo[k]) : 0.0;
      uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, t * 2097151.0));
      c |= spread21(q) << k;
    }
    key[d] = c;
  }
  std::vector<int32_t> order(nd);
  {
    std::vector<std::pair<uint64_t, int32_t>> kv(nd);
#pragma omp parallel for
    for (int64_t d = 0; d < nd; ++d) kv[d] = std::make_pair(key[d], (int32_t)d);
    __gnu_parallel::sort(kv.begin(), kv.end());  // by key, ties by dof id
#pragma omp parallel for
    for (int64_t d = 0; d < nd; ++d) order[d] = kv[d].second;
  }
  // blocks: contiguous runs of the Morton order, cut by prefix sums.  Row t has
  // weight w_t = max(len_t, 4) (so a block of weight <= kAccMax holds at most
  // kRowsMax rows); with W_t the exclusive prefix and W the total, row t goes to
  // block floor(W_t nbk / W), and every block weighs at most W / nbk + max w <=
  // kAccMax.  nbk is the smallest count that guarantees this, raised to a multiple
  // of the SM count (the kernel runs one persistent CTA per SM: no partial last
  // wave); blocks left empty by a heavy row are dropped.  The rule needs only a
  // scan, so the GPU build computes the same blocks.
  std::vector<int32_t> block_of(nd);
  std::vector<int64_t> bstart;  // into order
  {
    int64_t wtot = 0, wmax = 0;
    for (int64_t t = 0; t < nd; ++t) {
      const int64_t l = p->rowptr[order[t] + 1] - p->rowptr[order[t]];
      wtot += std::max<int64_t>(l, 4);
      wmax = std::max<int64_t>(wmax, std::max<int64_t>(l, 4));
    }
    const int64_t nbk = schedule_block_count(wtot, wmax, sm_count_hint());
    int64_t wex = 0, prev = -1;
    for (int64_t t = 0; t < nd; ++t) {
      const int64_t b = wex * nbk / wtot;
      if (b != prev) {
        bstart.push_back(t);
        prev = b;
      }
      block_of[order[t]] = (int32_t)bstart.size() - 1;
      wex += std::max<int64_t>(p->rowptr[order[t] + 1] - p->rowptr[order[t]], 4);
    }
  }
  bstart.push_back(nd);
  const int32_t nbk = (int32_t)bstart.size() - 1;
  // owned rows per block, ascending row id; accumulator base of each row
  std::vector<int32_t> row_acc_of(nd);
  hs->rows.resize(nd);
  hs->row_acc.resize(nd);
  hs->blocks.assign(nbk, BlockDesc{});
#pragma omp parallel for schedule(dynamic, 16)
  for (int32_t b = 0; b < nbk; ++b) {
    std::vector<int32_t> rs(order.begin() + bstart[b], order.begin() + bstart[b + 1]);
    std::sort(rs.begin(), rs.end());
    int32_t acc = 0;
    for (size_t k = 0; k < rs.size(); ++k) {
      hs->rows[bstart[b] + k] = rs[k];
      hs->row_acc[bstart[b] + k] = acc;
      row_acc_of[rs[k]] = acc;
      acc += p->rowptr[rs[k] + 1] - p->rowptr[rs[k]];
    }
    hs->blocks[b].row_begin = (int32_t)bstart[b];
    hs->blocks[b].row_count = (int32_t)(bstart[b + 1] - bstart[b]);
    hs->blocks[b].acc_used = acc;
  }
  // items: (block, element) for every block an element touches, element order
  std::vector<int64_t> bcount(nbk + 1, 0);
  auto blocks_of_elem = [&](int64_t e, int32_t* out) {
    int n = 0;
    for (int i = 0; i < nb; ++i) {
      int32_t b = block_of[m->dofs[e * nb + i]];
      bool seen = false;
      for (int u = 0; u < n; ++u) seen |= (out[u] == b);
      if (!seen) out[n++] = b;
    }
    return n;
  };
  {
    // per-thread counts over a static split of the elements, then each thread
    // fills its own ranges in the same split (each block's list is sorted below
    // by key, then element id)
    const int nth = std::max(1, omp_get_max_threads());
    std::vector<int64_t> tc((size_t)nth * nbk, 0);
#pragma omp parallel num_threads(nth)
    {
      int64_t* c = tc.data() + (size_t)omp_get_thread_num() * nbk;
#pragma omp for schedule(static)
      for (int64_t e = 0; e < E; ++e) {
        int32_t bs[10];
        const int n = blocks_of_elem(e, bs);
        for (int u = 0; u < n; ++u) c[bs[u]]++;
      }
    }
    for (int32_t b = 0; b < nbk; ++b) {
      int64_t at = bcount[b];
      for (int t = 0; t < nth; ++t) {
        const int64_t k = tc[(size_t)t * nbk + b];
        tc[(size_t)t * nbk + b] = at;
        at += k;
      }
      bcount[b + 1] = at;
    }
    if (bcount[nbk] >= INT32_MAX) return set_error(MG_ERR_SIZE, "assembly items above 2^31-1");
    hs->items.resize(bcount[nbk]);
#pragma omp parallel num_threads(nth)
    {
      int64_t* f = tc.data() + (size_t)omp_get_thread_num() * nbk;
#pragma omp for schedule(static)
      for (int64_t e = 0; e < E; ++e) {
        int32_t bs[10];
        const int n = blocks_of_elem(e, bs);
        for (int u = 0; u < n; ++u) hs->items[f[bs[u]]++] = (int32_t)e;
      }
    }
  }
  // order each block's items along the Morton curve of the element centroids, so
  // that a chunk covers a compact patch (its contributions to a CSR entry fall in
  // one segment, its vertices are neighbours in L2); ties by element id.  Then
  // pad every block's list to a multiple of 4 (16-byte aligned bulk copies).
  {
    std::vector<uint64_t> ekey(E);
#pragma omp parallel for
    for (int64_t e = 0; e < E; ++e) {
      double x[3] = {0, 0, 0};
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 3; ++k) x[k] += 0.25 * m->xyz[3 * (int64_t)m->conn[4 * e + v] + k];
      uint64_t c = 0;
      for (int k = 0; k < 3; ++k) {
        double t = hi[k] > lo[k] ? (x[k] - lo[k]) / (hi[k] - lo[k]) : 0.0;
        uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, t * 2097151.0));
        c |= spread21(q) << k;
      }
      ekey[e] = c;
    }
#pragma omp parallel
    {
      std::vector<std::pair<uint64_t, int32_t>> kv;
#pragma omp for schedule(dynamic, 16)
      for (int32_t b = 0; b < nbk; ++b) {
        kv.clear();
        for (int64_t k = bcount[b]; k < bcount[b + 1]; ++k) kv.emplace_back(ekey[hs->items[k]], hs->items[k]);
        std::sort(kv.begin(), kv.end());  // by key, ties by element id
        for (int64_t k = bcount[b]; k < bcount[b + 1]; ++k) hs->items[k] = kv[k - bcount[b]].second;
      }
    }
    // the same order over all elements, for the per-element kernels (adjoint)
    {
      std::vector<std::pair<uint64_t, int32_t>> kv(E);
#pragma omp parallel for
      for (int64_t e = 0; e < E; ++e) kv[e] = std::make_pair(ekey[e], (int32_t)e);
      __gnu_parallel::sort(kv.begin(), kv.end());
      hs->elem_order.resize(E);
#pragma omp parallel for
      for (int64_t e = 0; e < E; ++e) hs->elem_order[e] = kv[e].second;
    }
    std::vector<int32_t> padded;
    padded.reserve(hs->items.size() + 4 * (size_t)nbk);
    for (int32_t b = 0; b < nbk; ++b) {
      const int64_t i0 = bcount[b], i1 = bcount[b + 1];
      hs->blocks[b].item_begin = (int32_t)padded.size();
      hs->blocks[b].item_count = (int32_t)(i1 - i0);
      for (int64_t k = i0; k < i1; ++k) padded.push_back(hs->items[k]);
      while (padded.size() % 4) padded.push_back(-1);
    }
    if ((int64_t)padded.size() >= INT32_MAX) return set_error(MG_ERR_SIZE, "assembly items above 2^31-1");
    hs->items.swap(padded);
  }
  int64_t nchunk_tot = 0;
  for (int32_t b = 0; b < nbk; ++b) {
    BlockDesc& d = hs->blocks[b];
    d.chunk_begin = (int32_t)nchunk_tot;
    d.nchunks = (d.item_count + CI - 1) / CI;
    nchunk_tot += d.nchunks;
  }
  // chunk vertex tables: the distinct vertices of each chunk's elements in
  // first-appearance order (padded to a multiple of 4 with the chunk's first
  // vertex) and each item's local vertex indices
  {
    hs->chunk_node_begin.assign(nchunk_tot, 0);
    hs->chunk_n_nodes.assign(nchunk_tot, 0);
    hs->item_lconn.assign(hs->items.size() * 4, 0);
    std::vector<std::vector<int32_t>> cn(nchunk_tot);
    int32_t maxn = 0;
#pragma omp parallel reduction(max : maxn)
    {
      std::vector<int32_t> stamp(N, -1), local(N, 0);
#pragma omp for schedule(dynamic, 4)
      for (int32_t b = 0; b < nbk; ++b) {
        const BlockDesc& d = hs->blocks[b];
        for (int32_t c = 0; c < d.nchunks; ++c) {
          const int32_t ck = d.chunk_begin + c;
          auto& v = cn[ck];
          const int32_t i0 = c * CI, i1 = std::min(d.item_count, i0 + CI);
          for (int32_t it = i0; it < i1; ++it) {
            const int64_t slot = (int64_t)d.item_begin + it;
            const int64_t e = hs->items[slot];
            for (int k = 0; k < 4; ++k) {
              const int32_t nd = m->conn[4 * e + k];
              if (stamp[nd] != ck) {
                stamp[nd] = ck;
                local[nd] = (int32_t)v.size();
                v.push_back(nd);
              }
              hs->item_lconn[4 * slot + k] = (uint16_t)local[nd];
            }
          }
          while (v.size() % 4) v.push_back(v.empty() ? 0 : v[0]);
          maxn = std::max(maxn, (int32_t)v.size());
        }
      }
    }
    if (maxn > 65535) return set_error(MG_ERR_SIZE, "a chunk touches more than 65535 vertices");
    int64_t tot = 0;
    for (int64_t ck = 0; ck < nchunk_tot; ++ck) {
      if (tot >= INT32_MAX) return set_error(MG_ERR_SIZE, "chunk vertex records above 2^31-1");
      hs->chunk_node_begin[ck] = (int32_t)tot;
      hs->chunk_n_nodes[ck] = (int32_t)cn[ck].size();
      tot += (int64_t)cn[ck].size();
    }
    hs->chunk_nodes.resize(tot);
    for (int64_t ck = 0; ck < nchunk_tot; ++ck)
      std::copy(cn[ck].begin(), cn[ck].end(), hs->chunk_nodes.begin() + hs->chunk_node_begin[ck]);
    hs->max_chunk_nodes = maxn;
    p->max_chunk_nodes = maxn;
    // largest chunk record (layout at ChunkDesc)
    int64_t maxb = 0;
    for (int32_t b = 0; b < nbk; ++b)
      for (int32_t c = 0; c < hs->blocks[b].nchunks; ++c) {
        const int64_t n4 = (std::min(CI, hs->blocks[b].item_count - c * CI) + 3) & ~3;
        maxb = std::max(maxb, (int64_t)sizeof(ChunkDesc) + 12 * n4 + 36 * (int64_t)hs->chunk_n_nodes[hs->blocks[b].chunk_begin + c]);
      }
    if (maxb >= INT32_MAX) return set_error(MG_ERR_SIZE, "chunk record above 2 GiB");
    p->max_rec_bytes = (int32_t)maxb;
  }
  // contribution lists, per block in parallel, then concatenated
  const int nu = nunique(m->order);
  const uint32_t zero_src = (uint32_t)(nu * CI);
  if (zero_src > (m->order == 1 ? kP1SrcMask : kSrcMask))
    return set_error(MG_ERR_SIZE, "chunk buffer above the source index width");
  if (kAccMax + 1 > (int)kSlotMask + 1) return set_error(MG_ERR_SIZE, "accumulator above the 14-bit slot index");
  const int PW = piece_srcs(m->order);
  // one 8-byte piece: PW sources of one slot (layout at piece_srcs)
  auto make_piece = [&](uint32_t slot, const uint32_t* src) -> uint64_t {
    if (PW == 4)
      return (uint64_t)src[0] | (uint64_t)src[1] << kP1SrcBits | (uint64_t)src[2] << (2 * kP1SrcBits) |
             (uint64_t)src[3] << (3 * kP1SrcBits) | (uint64_t)slot << kP1SlotShift;
    const uint64_t w0 = src[0] | slot << kSrcBits, w1 = src[1] | slot << kSrcBits;
    return w0 | w1 << 32;
  };
  uint64_t pad_piece;
  {
    const uint32_t z[4] = {zero_src, zero_src, zero_src, zero_src};
    pad_piece = make_piece((uint32_t)kAccMax, z);
  }
  std::vector<std::vector<uint32_t>> ent(nbk);
  std::vector<std::vector<int64_t>> cptr(nbk);
  std::vector<int64_t> contrib(nbk, 0), maxc(nbk, 0);
#pragma omp parallel
  {
    struct Seg { int32_t slot, begin, len; };
    std::vector<std::vector<uint64_t>> per(kThreads);
    std::vector<std::vector<int32_t>> tseg(kThreads);
    std::vector<std::pair<int32_t, uint32_t>> list, tmp;  // (slot, src) in item order
    std::vector<Seg> segs, segs_by_len;
    std::vector<uint32_t> srcs;
    std::vector<int32_t> cnt;
#pragma omp for schedule(dynamic, 1)
    for (int32_t b = 0; b < nbk; ++b) {
      const BlockDesc& d = hs->blocks[b];
      for (int32_t c = 0; c < d.nchunks; ++c) {
        list.clear();
        const int32_t i0 = c * CI, i1 = std::min(d.item_count, i0 + CI);
        for (int32_t it = i0; it < i1; ++it) {
          const int64_t e = hs->items[d.item_begin + it];
          const int32_t t = it - i0;
          for (int i = 0; i < nb; ++i) {      // field (column)
            const int32_t col = m->dofs[e * nb + i];
            for (int j = 0; j < nb; ++j) {    // test (row)
              const int32_t row = m->dofs[e * nb + j];
              if (block_of[row] != b) continue;
              // position of col in the row's sorted columns (rows are short:
              // a branch-free count beats a binary search)
              const int32_t* c0 = p->colind.data() + p->rowptr[row];
              const int32_t len = p->rowptr[row + 1] - p->rowptr[row];
              int32_t pos = 0;
              for (int32_t k = 0; k < len; ++k) pos += c0[k] < col;
              const int32_t acc = row_acc_of[row] + pos;
              list.emplace_back(acc, (uint32_t)(sym_index(i, j, nb) * CI + t));
            }
          }
        }
        contrib[b] += (int64_t)list.size();
        // segments: one per slot, contributions kept in item (= element) order --
        // a stable sort by slot (< 2^14: two 7-bit counting passes)
        tmp.resize(list.size());
        for (int pass = 0; pass < 2; ++pass) {
          const int sh = 7 * pass;
          cnt.assign(129, 0);
          for (const auto& x : list) cnt[((x.first >> sh) & 127) + 1]++;
          for (int k = 0; k < 128; ++k) cnt[k + 1] += cnt[k];
          for (const auto& x : list) tmp[cnt[(x.first >> sh) & 127]++] = x;
          list.swap(tmp);
        }
        segs.clear();
        srcs.clear();
        for (size_t k = 0; k < list.size(); ++k) {
          if (k == 0 || list[k].first != list[k - 1].first) segs.push_back({list[k].first, (int32_t)k, 0});
          segs.back().len++;
          srcs.push_back(list[k].second);
        }
        // longest segment first (a stable counting sort by length, descending),
        // to the least-loaded thread (ties: lowest thread)
        {
          int32_t maxlen = 0;
          for (const Seg& sg : segs) maxlen = std::max(maxlen, sg.len);
          cnt.assign(maxlen + 2, 0);
          for (const Seg& sg : segs) cnt[maxlen - sg.len + 1]++;
          for (int32_t k = 0; k <= maxlen; ++k) cnt[k + 1] += cnt[k];
          segs_by_len.resize(segs.size());
          for (const Seg& sg : segs) segs_by_len[cnt[maxlen - sg.len]++] = sg;
          segs.swap(segs_by_len);
        }
        // dealt in snake order of that ranking: rank q goes to thread q mod T
        // on even rounds (q / T) and T - 1 - q mod T on odd ones, which gives
        // each thread nearly the same load and each warp lanes of similar loads
        for (auto& v : tseg) v.clear();
        for (size_t q = 0; q < segs.size(); ++q) {
          const int r = (int)(q / kThreads), o = (int)(q % kThreads);
          tseg[(r & 1) ? kThreads - 1 - o : o].push_back((int32_t)q);
        }
        // each thread's segments cut into pieces of PW sources (the last piece
        // of a segment padded with the zero source); pieces keep element order
        for (int t = 0; t < kThreads; ++t) {
          auto& v = per[t];
          v.clear();
          for (int32_t q : tseg[t]) {
            const Seg& sg = segs[q];
            for (int k0 = 0; k0 < sg.len; k0 += PW) {
              uint32_t src[4];
              for (int k = 0; k < PW; ++k) src[k] = k0 + k < sg.len ? srcs[sg.begin + k0 + k] : zero_src;
              v.push_back(make_piece((uint32_t)sg.slot, src));
            }
          }
        }
        const int64_t base = (int64_t)ent[b].size();
        for (int w = 0; w < kWarps; ++w) {
          cptr[b].push_back((int64_t)ent[b].size());
          size_t K = 0;  // pieces
          for (int l = 0; l < 32; ++l) K = std::max(K, per[32 * w + l].size());
          // layout [piece][lane]: one 8-byte load per lane and piece (two words, lower first)
          for (size_t k = 0; k < K; ++k)
            for (int l = 0; l < 32; ++l) {
              const auto& v = per[32 * w + l];
              const uint64_t pc = k < v.size() ? v[k] : pad_piece;
              ent[b].push_back((uint32_t)pc);
              ent[b].push_back((uint32_t)(pc >> 32));
            }
        }
        cptr[b].push_back((int64_t)ent[b].size());
        maxc[b] = std::max(maxc[b], (int64_t)ent[b].size() - base);
      }
    }
  }
  int64_t total = 0;
  for (int32_t b = 0; b < nbk; ++b) total += (int64_t)ent[b].size();
  hs->entries.resize(total);
  hs->chunk_ptr.resize(nchunk_tot * (kWarps + 1));
  std::vector<int64_t> boff(nbk + 1, 0);
  for (int32_t b = 0; b < nbk; ++b) {
    boff[b + 1] = boff[b] + (int64_t)ent[b].size();
    if (boff[b] % 32 != 0 || boff[b] / 32 >= INT32_MAX) return set_error(MG_ERR_SIZE, "contribution words above 2^36");
    hs->blocks[b].word_begin32 = (int32_t)(boff[b] / 32);
    hs->n_contrib += contrib[b];
    hs->max_chunk_entries = std::max(hs->max_chunk_entries, maxc[b]);
  }
#pragma omp parallel for schedule(dynamic, 4)
  for (int32_t b = 0; b < nbk; ++b) {
    std::copy(ent[b].begin(), ent[b].end(), hs->entries.begin() + boff[b]);
    const int64_t ck = hs->blocks[b].chunk_begin;
    for (size_t k = 0; k < cptr[b].size(); ++k) hs->chunk_ptr[ck * (kWarps + 1) + k] = cptr[b][k] + boff[b];
    std::vector<uint32_t>().swap(ent[b]);
  }
  // blocks stay in Morton order of their rows (the work counter hands them out
  // in array order): the blocks in flight at one time are neighbours, so the
  // coefficients of the elements they share are read from L2; the cut by
  // weight makes them nearly equal, so no longest-first order is needed
  p->nblocks = nbk;
  p->n_items = 0;
  for (int32_t b = 0; b < nbk; ++b) p->n_items += hs->blocks[b].item_count;
  p->n_item_slots = (int64_t)hs->items.size();
  p->n_chunks = nchunk_tot;
  p->n_entries = total;
  p->n_contrib = hs->n_contrib;
  p->max_chunk_entries = hs->max_chunk_entries;
  return MG_OK;
}

template <typename T>
static mg_status upload(T** dst, const std::vector<T>& src)
{
  MG_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
  if (!src.empty()) MG_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return MG_OK;
}

mg_status plan_device(mg_plan* p)
{
  if (p->on_device) return check_device(p->mesh->device, "the plan");
  std::lock_guard<std::mutex> lock(p->upload_mu);
  if (p->on_device) return check_device(p->mesh->device, "the plan");
  MG_TRY(mesh_device(p->mesh));
  const HostSchedule& hs = *p->host_schedule;
  MG_TRY(upload(&p->d_rowptr, p->rowptr));
  MG_TRY(upload(&p->d_colind, p->colind));
  std::vector<int32_t> diag(p->ndof);
  for (int64_t r = 0; r < p->ndof; ++r) {
    const int32_t* c0 = p->colind.data() + p->rowptr[r];
    const int32_t* c1 = p->colind.data() + p->rowptr[r + 1];
    diag[r] = p->rowptr[r] + (int32_t)(std::lower_bound(c0, c1, (int32_t)r) - c0);
  }
  MG_TRY(upload(&p->d_diag, diag));
  {
    // 16-bit column offsets (col - row) when every entry fits: 2 bytes per entry
    // less for the SpMV and CG kernels; the CSR arrays stay the reference's
    bool fits = true;
    std::vector<int16_t> off(p->colind.size());
#pragma omp parallel for reduction(&& : fits)
    for (int64_t r = 0; r < p->ndof; ++r)
      for (int32_t k = p->rowptr[r]; k < p->rowptr[r + 1]; ++k) {
        const int64_t d = (int64_t)p->colind[k] - r;
        if (d < INT16_MIN || d > INT16_MAX) fits = false;
        else off[k] = (int16_t)d;
      }
    if (fits && !off.empty()) MG_TRY(upload(&p->d_coloff, off));
  }
  MG_TRY(upload(&p->d_blocks, hs.blocks));
  MG_TRY(upload(&p->d_entries, hs.entries));
  {
    const int nb = p->mesh->nb;
    std::vector<int32_t> dm((size_t)hs.elem_order.size() * nb);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)hs.elem_order.size(); ++i)
      for (int k = 0; k < nb; ++k) dm[i * nb + k] = p->mesh->dofs[(int64_t)hs.elem_order[i] * nb + k];
    MG_TRY(upload(&p->d_elem_order, hs.elem_order));
    MG_TRY(upload(&p->d_dofs_morton, dm));
  }
  {
    // owned-row metadata in schedule order, padded by two entries so that the
    // kernel's 16-byte aligned copies of a row range stay inside the array
    std::vector<int2> meta(hs.rows.size() + 2, make_int2(0, 0));
    for (size_t k = 0; k < hs.rows.size(); ++k)
      meta[k] = make_int2(hs.row_acc[k], p->rowptr[hs.rows[k]] - hs.row_acc[k]);
    MG_TRY(upload(&p->d_row_meta, meta));
  }
  {
    // chunk records (layout at ChunkDesc): sizes, offsets, then the contents
    const int CI = chunk_items(p->mesh->order);
    const int64_t nc = (int64_t)hs.chunk_ptr.size() / (kWarps + 1);
    std::vector<int32_t> blk(nc), pos(nc);  // owning block, chunk index within it
    for (size_t b = 0; b < hs.blocks.size(); ++b)
      for (int32_t c = 0; c < hs.blocks[b].nchunks; ++c) {
        blk[hs.blocks[b].chunk_begin + c] = (int32_t)b;
        pos[hs.blocks[b].chunk_begin + c] = c;
      }
    auto n_items = [&](int64_t ck) {
      const BlockDesc& d = hs.blocks[blk[ck]];
      return std::min(CI, d.item_count - pos[ck] * CI);
    };
    std::vector<int2> rec(nc);
    std::vector<int64_t> off(nc + 1, 0);
    int64_t maxb = 0;
    for (int64_t ck = 0; ck < nc; ++ck) {
      const int64_t n4 = (n_items(ck) + 3) & ~3, nn = hs.chunk_n_nodes[ck];
      const int64_t bytes = (int64_t)sizeof(ChunkDesc) + 12 * n4 + 36 * nn;
      off[ck + 1] = off[ck] + bytes;
      maxb = std::max(maxb, bytes);
    }
    if (off[nc] / 16 >= INT32_MAX || maxb >= INT32_MAX)
      return set_error(MG_ERR_SIZE, "chunk records above 32 GiB");
    for (int64_t ck = 0; ck < nc; ++ck) rec[ck] = make_int2((int32_t)(off[ck] / 16), (int32_t)(off[ck + 1] - off[ck]));
    std::vector<unsigned char> data(std::max<int64_t>(off[nc], 16), 0);
    const std::vector<double>& xyz = p->mesh->xyz;
    std::vector<int32_t> rank_of(hs.elem_order.size());
    for (size_t i = 0; i < hs.elem_order.size(); ++i) rank_of[hs.elem_order[i]] = (int32_t)i;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t ck = 0; ck < nc; ++ck) {
      unsigned char* r = data.data() + off[ck];
      const BlockDesc& d = hs.blocks[blk[ck]];
      const int32_t c = pos[ck];
      const int64_t n4 = (n_items(ck) + 3) & ~3, nn = hs.chunk_n_nodes[ck];
      ChunkDesc cd{};
      const int64_t* cp = &hs.chunk_ptr[ck * (kWarps + 1)];
      cd.word_begin = cp[0];
      for (int w = 0; w <= kWarps; ++w) cd.warp_off[w] = (int32_t)(cp[w] - cp[0]);
      cd.n_nodes = (int32_t)nn;
      if (c + kRecStages < d.nchunks) {
        cd.next_off16 = rec[ck + kRecStages].x;
        cd.next_bytes = rec[ck + kRecStages].y;
      }
      std::memcpy(r, &cd, sizeof cd);
      const int64_t first = (int64_t)d.item_begin + (int64_t)c * CI;
      // the items' Morton ranks (the kernel reads the coefficient in that order)
      int32_t* ranks = reinterpret_cast<int32_t*>(r + 64);
      for (int64_t i = 0; i < n4; ++i) {
        const int32_t e = hs.items[first + i];
        ranks[i] = e >= 0 ? rank_of[e] : -1;
      }
      std::memcpy(r + 64 + 4 * n4, &hs.item_lconn[4 * first], 8 * n4);
      float4* va = reinterpret_cast<float4*>(r + 64 + 12 * n4);
      float4* vb = reinterpret_cast<float4*>(r + 64 + 12 * n4 + 16 * nn);
      float* vc = reinterpret_cast<float*>(r + 64 + 12 * n4 + 32 * nn);
      const int64_t n0 = hs.chunk_nodes[hs.chunk_node_begin[ck]];  // origin: the chunk's first vertex
      for (int64_t i = 0; i < nn; ++i) {
        // r = x - origin (FP64), then r = hi + mid + lo exactly: hi = fl(r),
        // mid = fl(r - hi), lo = r - hi - mid (each remainder exact in FP64)
        const int64_t nd = hs.chunk_nodes[hs.chunk_node_begin[ck] + i];
        float h[3], md[3], l[3];
        for (int k = 0; k < 3; ++k) {
          const double rr = xyz[3 * nd + k] - xyz[3 * n0 + k];
          h[k] = (float)rr;
          const double r1 = rr - (double)h[k];
          md[k] = (float)r1;
          l[k] = (float)(r1 - (double)md[k]);
        }
        va[i] = make_float4(h[0], h[1], h[2], md[0]);
        vb[i] = make_float4(md[1], md[2], l[0], l[1]);
        vc[i] = l[2];
      }
    }
    MG_TRY(upload(&p->d_chunk_data, data));
    MG_TRY(upload(&p->d_chunk_rec, rec));
    // first word of each chunk (chunks are contiguous in the word array)
    std::vector<int64_t> wb(nc + 1, 0);
    for (int64_t ck = 0; ck < nc; ++ck) wb[ck] = hs.chunk_ptr[ck * (kWarps + 1)];
    wb[nc] = (int64_t)hs.entries.size();
    MG_TRY(upload(&p->d_chunk_wb, wb));
    if (maxb != p->max_rec_bytes) return set_error(MG_ERR_SIZE, "chunk record size mismatch");
  }
  MG_TRY(upload(&p->d_counters, std::vector<uint32_t>(8, 0u)));
  MG_CUDA(cudaMallocHost(&p->h_pinned, 64 * sizeof(double)));
  p->h_elem_order.swap(p->host_schedule->elem_order);  // kept for the load-vector map
  delete p->host_schedule;
  p->host_schedule = nullptr;
  p->on_device = true;
  return MG_OK;
}

static void free_plan(mg_plan* p)
{
  if (!p) return;
  cudaFree(p->d_rowptr);
  cudaFree(p->d_colind);
  cudaFree(p->d_diag);
  cudaFree(p->d_coloff);
  cudaFree(p->d_blocks);
  cudaFree(p->d_chunk_data);
  cudaFree(p->d_chunk_rec);
  cudaFree(p->d_chunk_wb);
  cudaFree(p->d_row_meta);
  cudaFree(p->d_sched_rows);
  cudaFree(p->d_elem_order);
  cudaFree(p->d_coeff_m);
  cudaFree(p->d_dofs_morton);
  cudaFree(p->d_rhs_ptr);
  cudaFree(p->d_rhs_slot);
  cudaFree(p->d_rhs_y);
  cudaFree(p->d_geo_det);
  cudaFree(p->d_geo_cof);
  cudaFree(p->d_entries);
  cudaFree(p->d_counters);
  for (double* t : p->d_tables) cudaFree(t);
  cudaFree(p->d_work);
  cudaFree(p->d_tmp_values);
  cudaFree(p->d_tmp_coeff);
  if (p->h_pinned) cudaFreeHost(p->h_pinned);
  delete p->host_schedule;
  delete p;
}

mg_status plan_tables(mg_plan* p, int quad, const RefTables** t, const double** d_tab)
{
  for (size_t k = 0; k < p->tables.size(); ++k)
    if (p->tables[k].quad == quad) {
      *t = &p->tables[k];
      *d_tab = p->d_tables[k];
      return MG_OK;
    }
  RefTables rt;
  MG_TRY(build_ref_tables(p->mesh->order, quad, &rt));
  // device layout: unique (i <= j, sym_index order) entries, stiff[6][nu] then mass[nu]
  const int nb = rt.nb, nu = nb * (nb + 1) / 2;
  std::vector<double> flat(7 * nu);
  for (int i = 0; i < nb; ++i)
    for (int j = i; j < nb; ++j) {
      const int u = sym_index(i, j, nb);
      for (int q = 0; q < 6; ++q) flat[q * nu + u] = rt.stiff[q * nb * nb + i * nb + j];
      flat[6 * nu + u] = rt.mass[i * nb + j];
    }
  double* d = nullptr;
  MG_CUDA(cudaMalloc(&d, sizeof(double) * flat.size()));
  MG_CUDA(cudaMemcpy(d, flat.data(), sizeof(double) * flat.size(), cudaMemcpyHostToDevice));
  p->tables.push_back(rt);
  p->d_tables.push_back(d);
  *t = &p->tables.back();
  *d_tab = d;
  return MG_OK;
}

// Load-vector map: for each dof (natural order), the element-vector slots
// q = p * nb + l with dofs_morton[q] == dof, ascending -- the fixed order in
// which the gather kernel sums them.  A parallel counting transpose, then each
// dof's short list sorted.
mg_status plan_rhs_map(mg_plan* p)
{
  if (p->d_rhs_ptr) return MG_OK;
  const mg_mesh* m = p->mesh;
  const int nb = m->nb;
  const int64_t E = m->n_elem, nd = p->ndof, pairs = E * nb;
  if (pairs >= INT32_MAX) return set_error(MG_ERR_SIZE, "load-vector map above 2^31 element-vector entries");
  if ((int64_t)p->h_elem_order.size() != E) return set_error(MG_ERR_INVALID_ARG, "plan without an element order");
  const int32_t* eo = p->h_elem_order.data();
  const int32_t* dofs = m->dofs.data();
  auto dof_of = [&](int64_t q) { return dofs[(int64_t)eo[q / nb] * nb + q % nb]; };
  std::vector<int32_t> ptr(nd + 1, 0), slot(std::max<int64_t>(pairs, 1));
#pragma omp parallel for
  for (int64_t q = 0; q < pairs; ++q) {
    const int32_t d = dof_of(q);
#pragma omp atomic
    ptr[d + 1]++;
  }
  for (int64_t d = 0; d < nd; ++d) ptr[d + 1] += ptr[d];
  std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
#pragma omp parallel for
  for (int64_t q = 0; q < pairs; ++q) {
    const int32_t d = dof_of(q);
    int32_t at;
#pragma omp atomic capture
    at = cur[d]++;
    slot[at] = (int32_t)q;
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t d = 0; d < nd; ++d) std::sort(slot.begin() + ptr[d], slot.begin() + ptr[d + 1]);
  // all three buffers or none (the map counts as built once d_rhs_ptr is set)
  int32_t *d_ptr = nullptr, *d_slot = nullptr;
  double* d_y = nullptr;
  mg_status st = upload(&d_ptr, ptr);
  if (st == MG_OK) st = upload(&d_slot, slot);
  if (st == MG_OK) {
    const cudaError_t e = cudaMalloc(&d_y, sizeof(double) * std::max<int64_t>(pairs, 1));
    if (e != cudaSuccess) st = cuda_error(e, "load-vector buffer");
  }
  if (st != MG_OK) {
    cudaFree(d_ptr);
    cudaFree(d_slot);
    cudaFree(d_y);
    return st;
  }
  p->d_rhs_ptr = d_ptr;
  p->d_rhs_slot = d_slot;
  p->d_rhs_y = d_y;
  return MG_OK;
}

mg_status plan_work(mg_plan* p, size_t bytes, void** ptr)
{
  if (p->work_bytes < bytes) {
    cudaFree(p->d_work);
    p->d_work = nullptr;
    p->work_bytes = 0;
    MG_CUDA(cudaMalloc(&p->d_work, bytes));
    p->work_bytes = bytes;
  }
  *ptr = p->d_work;
  return MG_OK;
}

}  // namespace mg

using namespace mg;

// The schedule of a plan built on the GPU, in the export format, read back from
// the device arrays (blocks, chunk records, words, row metadata).
static mg_status export_device_schedule(const mg_plan* p, int32_t* h_blocks, int32_t* h_items, int64_t* h_chunk_ptr,
                                        uint32_t* h_entries, int32_t* h_rows, int32_t* h_row_acc)
{
  const int CI = chunk_items(p->mesh->order);
  std::vector<BlockDesc> blocks(p->nblocks);
  if (p->nblocks) MG_CUDA(cudaMemcpy(blocks.data(), p->d_blocks, sizeof(BlockDesc) * p->nblocks, cudaMemcpyDeviceToHost));
  if (h_blocks) std::memcpy(h_blocks, blocks.data(), sizeof(BlockDesc) * blocks.size());
  if (h_entries && p->n_entries)
    MG_CUDA(cudaMemcpy(h_entries, p->d_entries, sizeof(uint32_t) * p->n_entries, cudaMemcpyDeviceToHost));
  if (h_rows && p->ndof) MG_CUDA(cudaMemcpy(h_rows, p->d_sched_rows, sizeof(int32_t) * p->ndof, cudaMemcpyDeviceToHost));
  if (h_row_acc && p->ndof) {
    std::vector<int2> meta(p->ndof);
    MG_CUDA(cudaMemcpy(meta.data(), p->d_row_meta, sizeof(int2) * p->ndof, cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < p->ndof; ++k) h_row_acc[k] = meta[k].x;
  }
  if (h_items || h_chunk_ptr) {
    std::vector<int2> rec(p->n_chunks);
    if (p->n_chunks) MG_CUDA(cudaMemcpy(rec.data(), p->d_chunk_rec, sizeof(int2) * p->n_chunks, cudaMemcpyDeviceToHost));
    const int64_t bytes = p->n_chunks ? (int64_t)rec.back().x * 16 + rec.back().y : 0;
    std::vector<unsigned char> data(std::max<int64_t>(bytes, 1));
    if (bytes) MG_CUDA(cudaMemcpy(data.data(), p->d_chunk_data, bytes, cudaMemcpyDeviceToHost));
    for (const BlockDesc& d : blocks)
      for (int32_t c = 0; c < d.nchunks; ++c) {
        const int64_t ck = d.chunk_begin + c;
        const unsigned char* r = data.data() + (int64_t)rec[ck].x * 16;
        ChunkDesc cd;
        std::memcpy(&cd, r, sizeof cd);
        if (h_chunk_ptr)
          for (int w = 0; w <= kWarps; ++w) h_chunk_ptr[ck * (kWarps + 1) + w] = cd.word_begin + cd.warp_off[w];
        const int n4 = (std::min(CI, d.item_count - c * CI) + 3) & ~3;
        if (h_items) {
          // the records hold Morton ranks: back to element ids
          const int32_t* rk = reinterpret_cast<const int32_t*>(r + sizeof(ChunkDesc));
          int32_t* out = h_items + d.item_begin + (int64_t)c * CI;
          for (int64_t i = 0; i < n4; ++i) out[i] = rk[i] >= 0 ? p->h_elem_order[rk[i]] : -1;
        }
      }
  }
  return MG_OK;
}

extern "C" {

mg_status mg_pattern_build(mg_mesh* mesh, mg_plan** out)
{
  NvtxRange nvtx_range("mg_pattern_build");
  if (!mesh || !out) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_build: null argument");
  *out = nullptr;
  mg_plan* p = new mg_plan();
  p->mesh = mesh;
  p->host_schedule = new HostSchedule();
  mg_status s = build_pattern(p);
  if (s == MG_OK) s = build_schedule(p, p->host_schedule);
  if (s != MG_OK) {
    free_plan(p);
    return s;
  }
  *out = p;
  return MG_OK;
}

mg_status mg_pattern_build_device(mg_mesh* mesh, mg_plan** out, void* stream)
{
  NvtxRange nvtx_range("mg_pattern_build_device");
  if (!mesh || !out) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_build_device: null argument");
  *out = nullptr;
  mg_plan* p = new mg_plan();
  p->mesh = mesh;
  mg_status s = build_pattern_device(p, (cudaStream_t)stream, true);
  if (s == MG_OK) s = build_schedule_device(p, (cudaStream_t)stream);
  if (s != MG_OK) {
    free_plan(p);
    return s;
  }
  *out = p;
  return MG_OK;
}

mg_status mg_plan_destroy(mg_plan* plan)
{
  free_plan(plan);
  return MG_OK;
}

mg_status mg_pattern_info(const mg_plan* p, int64_t* ndof, int64_t* nnz)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_info: null plan");
  if (ndof) *ndof = p->ndof;
  if (nnz) *nnz = p->nnz;
  return MG_OK;
}

mg_status mg_pattern_export(const mg_plan* p, int32_t* h_rowptr, int32_t* h_colind)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_export: null plan");
  if (h_rowptr) std::memcpy(h_rowptr, p->rowptr.data(), sizeof(int32_t) * p->rowptr.size());
  if (h_colind) std::memcpy(h_colind, p->colind.data(), sizeof(int32_t) * p->colind.size());
  return MG_OK;
}

mg_status mg_pattern_device(const mg_plan* pc, const int32_t** d_rowptr, const int32_t** d_colind)
{
  mg_plan* p = const_cast<mg_plan*>(pc);
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_pattern_device: null plan");
  MG_TRY(plan_device(p));
  if (d_rowptr) *d_rowptr = p->d_rowptr;
  if (d_colind) *d_colind = p->d_colind;
  return MG_OK;
}

mg_status mg_plan_schedule_info(const mg_plan* p, mg_schedule_info* info)
{
  if (!p || !info) return set_error(MG_ERR_INVALID_ARG, "mg_plan_schedule_info: null argument");
  info->nblocks = p->nblocks;
  info->threads = kThreads;
  info->warps = kWarps;
  info->acc_max = kAccMax;
  info->chunk_items = chunk_items(p->mesh->order);
  info->host_copy = p->host_schedule != nullptr || p->d_sched_rows != nullptr;
  info->n_items = p->n_items;
  info->n_chunks = p->n_chunks;
  info->n_entries = p->n_entries;
  info->n_contrib = p->n_contrib;
  info->n_item_slots = p->n_item_slots;
  info->max_chunk_entries = p->max_chunk_entries;
  info->max_chunk_vertices = p->max_chunk_nodes;
  info->max_chunk_record_bytes = p->max_rec_bytes;
  return MG_OK;
}

mg_status mg_plan_export_schedule(const mg_plan* p, int32_t* h_blocks, int32_t* h_items,
                                  int64_t* h_chunk_ptr, uint32_t* h_entries, int32_t* h_rows,
                                  int32_t* h_row_acc)
{
  if (!p) return set_error(MG_ERR_INVALID_ARG, "mg_plan_export_schedule: null plan");
  const HostSchedule* hs = p->host_schedule;
  static_assert(sizeof(BlockDesc) == 8 * sizeof(int32_t), "BlockDesc layout");
  if (!hs && p->d_sched_rows) return export_device_schedule(p, h_blocks, h_items, h_chunk_ptr, h_entries, h_rows, h_row_acc);
  if (!hs)
    return set_error(MG_ERR_UNSUPPORTED,
                     "the host copy of the schedule is released once the plan is used on the GPU");
  if (h_blocks) std::memcpy(h_blocks, hs->blocks.data(), sizeof(BlockDesc) * hs->blocks.size());
  if (h_items) std::memcpy(h_items, hs->items.data(), sizeof(int32_t) * hs->items.size());
  if (h_chunk_ptr) std::memcpy(h_chunk_ptr, hs->chunk_ptr.data(), sizeof(int64_t) * hs->chunk_ptr.size());
  if (h_entries) std::memcpy(h_entries, hs->entries.data(), sizeof(uint32_t) * hs->entries.size());
  if (h_rows) std::memcpy(h_rows, hs->rows.data(), sizeof(int32_t) * hs->rows.size());
  if (h_row_acc) std::memcpy(h_row_acc, hs->row_acc.data(), sizeof(int32_t) * hs->row_acc.size());
  return MG_OK;
}

}  // extern "C"
