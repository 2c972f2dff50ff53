// bf_search.cu — exact brute-force k-NN (BruteForceIndex::node_search_k,
// src/index/bruteforce_idx.rs:47-73) for a batch of queries.
//
// The base is scanned in a few large chunks.  The first chunk offers every
// row to the per-query k-best lists; each later chunk offers only rows whose
// (distance,row) key beats the query's current k-th key, which after the
// first chunk is already a tight bound, so the candidate traffic is a few
// thousand keys per query for the whole base.  Chunk sizes grow with the
// rows already seen so that the expected candidates per chunk stay near a
// quarter of the per-query capacity.  A query whose candidates overflow the
// capacity is rescanned over the whole base with its tightened bound until
// nothing overflows; duplicates from a rescan are dropped by the merge.  The
// result is the exact k smallest (distance,row) keys, independent of the
// chunking.
#include <algorithm>

#include "internal.h"

namespace hora {

static int stage_ws(SearchWorkspace &ws, int64_t nq, int k, int cap, cudaStream_t s) {
  HORA_TRY(ws.best.reserve(sizeof(uint64_t) * nq * k));
  HORA_TRY(ws.cand.reserve(sizeof(uint64_t) * nq * cap));
  HORA_TRY(ws.count.reserve(sizeof(uint32_t) * nq));
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(sizeof(uint32_t)));
  HORA_TRY(ws.qlist.reserve(sizeof(int) * nq));
  return HORA_OK;
}

int bf_topk_exact(const BaseView &b, int metric, const float *dQ, const float *dqnorm, int64_t nq,
                  int k, int cand_cap, SearchWorkspace &ws, uint64_t *d_best, cudaStream_t s,
                  int *retries_out) {
  if (retries_out) *retries_out = 0;
  if (nq <= 0) return HORA_OK;
  if (k <= 0) return fail(HORA_EINVAL, "k must be positive");
  int cap = std::max(cand_cap, 2 * k);
  cap = (int)round_up(cap, 128);
  HORA_TRY(stage_ws(ws, nq, k, cap, s));
  uint32_t *count = ws.count.as<uint32_t>();
  uint64_t *cand = ws.cand.as<uint64_t>();
  uint8_t *flags = ws.ovf_flag.as<uint8_t>();
  uint32_t *ovc = ws.ovf_counter.as<uint32_t>();
  HORA_CUDA_TRY(cudaMemsetAsync(d_best, 0xff, sizeof(uint64_t) * nq * k, s));
  HORA_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(uint32_t) * nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(flags, 0, nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(ovc, 0, sizeof(uint32_t), s));
  if (b.n == 0) return HORA_OK;

  TileParams p;
  p.Q = dQ;
  p.ldq = b.ld;
  p.nq = nq;
  p.X = b.X;
  p.ldx = b.ld;
  p.ld = b.ld;
  p.qnorm = dqnorm;
  p.xnorm = b.xnorm;
  p.best = d_best;
  p.k = k;
  p.cand = cand;
  p.cap = cap;
  p.count = count;

  // chunk 0: every row is a candidate
  int64_t c0 = std::min<int64_t>(b.n, std::min<int64_t>(cap, round_up(std::max(2 * k, 1024), 128)));
  p.r_begin = 0;
  p.r_end = c0;
  HORA_TRY(launch_dist_tile(metric, TILE_DENSE, p, s));
  HORA_TRY(launch_merge_topk(d_best, k, cand, count, cap, (int)c0, nullptr, nq, flags, ovc, s));
  int64_t done = c0;
  const int64_t max_chunk = (int64_t)65535 * 128;
  while (done < b.n) {
    double grow = (double)cap / (4.0 * k);
    int64_t c = (int64_t)((double)done * std::max(grow, 1.0));
    c = std::max<int64_t>(c, 128 * 64);
    c = std::min<int64_t>(round_up(c, 128), std::min<int64_t>(b.n - done, max_chunk));
    p.r_begin = done;
    p.r_end = done + c;
    HORA_TRY(launch_dist_tile(metric, TILE_FILTER, p, s));
    HORA_TRY(launch_merge_topk(d_best, k, cand, count, cap, 0, nullptr, nq, flags, ovc, s));
    done += c;
  }

  // rescan queries whose candidates overflowed, until none do
  uint32_t h_ovc = 0;
  HORA_CUDA_TRY(cudaMemcpyAsync(&h_ovc, ovc, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  int rounds = 0;
  while (h_ovc > 0) {
    if (++rounds > 64) return fail(HORA_ECUDA, "brute force: candidate overflow did not converge");
    ws.h_flags.resize(nq);
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.h_flags.data(), flags, nq, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> list;
    for (int64_t q = 0; q < nq; ++q)
      if (ws.h_flags[q]) list.push_back((int)q);
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.qlist.ptr, list.data(), sizeof(int) * list.size(),
                                  cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaMemsetAsync(flags, 0, nq, s));
    HORA_CUDA_TRY(cudaMemsetAsync(ovc, 0, sizeof(uint32_t), s));
    TileParams r = p;
    r.nq = (int64_t)list.size();
    r.qmap = ws.qlist.as<int>();
    for (int64_t lo = 0; lo < b.n; lo += max_chunk) {
      r.r_begin = lo;
      r.r_end = std::min<int64_t>(b.n, lo + max_chunk);
      HORA_TRY(launch_dist_tile(metric, TILE_FILTER, r, s));
      HORA_TRY(launch_merge_topk(d_best, k, cand, count, cap, 0, ws.qlist.as<int>(), r.nq, flags,
                                 ovc, s));
    }
    HORA_CUDA_TRY(cudaMemcpyAsync(&h_ovc, ovc, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (retries_out) *retries_out = rounds;
  return HORA_OK;
}

}  // namespace hora
