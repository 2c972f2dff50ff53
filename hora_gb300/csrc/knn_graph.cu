// knn_graph.cu — the all-pairs k-nearest-neighbour graph of a brute-force
// index (SSGIndex::build_knn_graph, src/index/ssg_idx.rs:69-98): for every
// stored row, its k nearest other rows under the index metric.  It is the
// brute-force search with the base's own rows as queries (in the index's
// precision: exact FP32, or BF16 / FP8 scoring with the exact rerank), k + 1
// results per row and the row itself dropped.  The reference leaves each
// list in max-heap pop order (farthest first); so does this.
#include <algorithm>
#include <vector>

#include "index.h"

using namespace hora;

extern "C" {

int hora_knn_graph(hora_index *h, uint64_t k, uint64_t *neighbors_out) {
  if (!h || !neighbors_out) return fail(HORA_EINVAL, "null argument");
  if (h->kind != HORA_INDEX_BRUTE_FORCE) return fail(HORA_EINVAL, "the kNN graph is built on a BruteForceIndex");
  std::lock_guard<std::mutex> g(h->mu);
  if (!h->built || h->metric == HORA_METRIC_UNKNOWN) return fail(HORA_ENOTBUILT, "index not built");
  const int64_t n = h->n;
  if (k == 0 || (int64_t)k >= n) return fail(HORA_EINVAL, "k must be in [1, n - 1]");
  if (k + 1 > 4096) return fail(HORA_ECAP, "k must be < 4096");
  cudaStream_t s = h->stream;
  SearchWorkspace &ws = h->ws;
  const int kk = (int)k + 1;
  const int64_t B = 8192;  // query rows per batch
  DevBuf rows;
  HORA_TRY(rows.reserve(sizeof(float) * std::min<int64_t>(B, n) * h->dim));
  HORA_TRY(ws.keys2.reserve(sizeof(uint64_t) * std::min<int64_t>(B, n) * kk));
  std::vector<uint64_t> keys((size_t)std::min<int64_t>(B, n) * kk);
  for (int64_t b0 = 0; b0 < n; b0 += B) {
    const int64_t nb = std::min<int64_t>(B, n - b0);
    // the batch's rows, unpadded, as the queries
    HORA_CUDA_TRY(cudaMemcpy2DAsync(rows.ptr, h->dim * 4, h->base.as<float>() + b0 * h->ld, h->ld * 4,
                                    h->dim * 4, nb, cudaMemcpyDeviceToDevice, s));
    HORA_TRY(stage_queries(h, rows.as<float>(), nb, ws, s));
    HORA_TRY(bf_search_keys(h, nb, kk, ws, ws.keys2.as<uint64_t>(), s));
    HORA_CUDA_TRY(cudaMemcpyAsync(keys.data(), ws.keys2.ptr, sizeof(uint64_t) * nb * kk,
                                  cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < nb; ++i) {
      const uint64_t self = (uint64_t)(b0 + i);
      const uint64_t *kq = keys.data() + i * kk;
      uint64_t *o = neighbors_out + (b0 + i) * k;
      // ascending keys without the row itself (or without the last one when
      // the row is not among them: more than k exact duplicates), written
      // farthest first
      int w = 0;
      bool dropped = false;
      for (int j = 0; j < kk && w < (int)k; ++j) {
        const uint64_t r = key_row(kq[j]);
        if (!dropped && r == self) {
          dropped = true;
          continue;
        }
        o[k - 1 - w] = kq[j] == kEmptyKey ? HORA_NO_ID : r;
        ++w;
      }
    }
  }
  return HORA_OK;
}

}  // extern "C"
