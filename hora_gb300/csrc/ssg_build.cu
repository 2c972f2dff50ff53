// ssg_build.cu — the data-parallel steps of SSGIndex's build
// (src/index/ssg_idx.rs) on a built brute-force index.
//
// hora_knn_graph: build_knn_graph (ssg_idx.rs:69-98), for every stored row
// its k nearest other rows under the index metric.  It is the brute-force
// search with the base's own rows as queries (in the index's precision: exact
// FP32, or BF16 / FP8 scoring with the exact rerank), k + 1 results per row
// and the row itself dropped.  The reference leaves each list in max-heap pop
// order (farthest first); so does this.
//
// hora_general_kmeans: kmeans::general_kmeans (src/core/kmeans.rs:216-289),
// the root selection of ssg_idx.rs:388.  k means start as copies of k rows
// (drawn with replacement); each epoch assigns every row to its nearest mean
// (strict '<' from f32::MAX, so ties go to the lower mean and a row with no
// distance below f32::MAX stays with mean 0), then replaces each mean by the
// f32 sum of its rows divided by their count (an empty mean becomes 0/0 =
// NaN, as in the reference).  The roots are, per mean, the row nearest to it
// under the same rule.  Distances are the exact FP32 direct forms; the sums
// run in row order (the order a single rayon thread takes; the reference's
// lock order varies from run to run).
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <vector>

#include "index.h"

using namespace hora;

namespace {

constexpr int64_t kMaxMeans = 32768;

// rows[i] of the base -> means[i] (pitch ld); the caller zeroed the padding
__global__ void gk_gather_kernel(const float *X, int64_t ld, int64_t dim, const uint64_t *rows, int64_t k,
                                 float *means) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= k * dim) return;
  const int64_t i = t / dim, j = t % dim;
  means[i * ld + j] = X[(int64_t)rows[i] * ld + j];
}

// smallest (distance, index) key -> index, or 0 when the distance is not
// below f32::MAX (the reference's incumbent starts at index 0, f32::MAX)
__global__ void gk_pick_kernel(const uint64_t *keys, int64_t n, uint32_t *labels, uint64_t *rows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = keys[i];
  const uint32_t r = key_dist(key) < FLT_MAX ? key_row(key) : 0u;
  if (labels) labels[i] = r;
  if (rows) rows[i] = r;
}

}  // namespace

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

int hora_general_kmeans(hora_index *h, uint64_t k, uint64_t epoch, const uint64_t *init_rows, uint64_t seed,
                        uint64_t *roots_out, float *means_out) {
  if (!h || !roots_out) return fail(HORA_EINVAL, "null argument");
  if (h->kind != HORA_INDEX_BRUTE_FORCE) return fail(HORA_EINVAL, "general_kmeans runs on a BruteForceIndex");
  std::lock_guard<std::mutex> g(h->mu);
  if (!h->built || h->metric == HORA_METRIC_UNKNOWN) return fail(HORA_ENOTBUILT, "index not built");
  const int64_t n = h->n;
  if (n == 0) return HORA_OK;  // the reference returns no roots
  if (k == 0) return fail(HORA_EINVAL, "k must be at least 1");
  if ((int64_t)k > kMaxMeans) return fail(HORA_ECAP, "k must be <= 32768");
  if (epoch > (uint64_t)1 << 20) return fail(HORA_EINVAL, "epoch out of range");
  const int64_t K = (int64_t)k, ld = h->ld, dim = h->dim;
  std::vector<uint64_t> rows((size_t)K);
  if (init_rows) {
    for (int64_t i = 0; i < K; ++i) {
      if (init_rows[i] >= (uint64_t)n) return fail(HORA_EINVAL, "init row out of range");
      rows[i] = init_rows[i];
    }
  } else {
    // rng.gen_range(0..n) per mean (kmeans.rs:228-230) from the seeded stream
    uint64_t st = instance_seed(seed, 0);
    for (int64_t i = 0; i < K; ++i) {
      st += kRngStep;
      rows[i] = (uint64_t)(((unsigned __int128)mix64(st) * (uint64_t)n) >> 64);
    }
  }
  cudaStream_t s = h->stream;
  const float *X = h->base.as<float>();
  DevBuf d_rows, means, cnorm, keys, labels, blk, cnt, off, members, best;
  HORA_TRY(d_rows.reserve(sizeof(uint64_t) * K));
  HORA_TRY(means.reserve(sizeof(float) * K * ld));
  HORA_TRY(cnorm.reserve(sizeof(float) * K));
  HORA_TRY(keys.reserve(sizeof(uint64_t) * n));
  HORA_TRY(labels.reserve(sizeof(uint32_t) * n));
  HORA_TRY(off.reserve(sizeof(int64_t) * (K + 1)));
  HORA_TRY(members.reserve(sizeof(uint32_t) * n));
  HORA_TRY(best.reserve(sizeof(uint64_t) * K));
  HORA_CUDA_TRY(cudaMemcpyAsync(d_rows.ptr, rows.data(), sizeof(uint64_t) * K, cudaMemcpyHostToDevice, s));
  HORA_CUDA_TRY(cudaMemsetAsync(means.ptr, 0, sizeof(float) * K * ld, s));
  gk_gather_kernel<<<ceil_div(K * dim, 256), 256, 0, s>>>(X, ld, dim, d_rows.as<uint64_t>(), K,
                                                          means.as<float>());
  HORA_LAUNCHED();
  const bool cos = h->metric == M_COS;
  if (cos) HORA_TRY(ensure_norms(h, s));
  for (uint64_t ep = 0; ep < epoch; ++ep) {
    if (cos) HORA_TRY(launch_row_norms(means.as<float>(), K, ld, dim, cnorm.as<float>(), nullptr, s));
    TileParams p;
    p.Q = X;
    p.ldq = ld;
    p.nq = n;
    p.X = means.as<float>();
    p.ldx = ld;
    p.r_begin = 0;
    p.r_end = K;
    p.ld = ld;
    p.qnorm = h->xnorm.as<float>();
    p.xnorm = cnorm.as<float>();
    p.out_key = keys.as<uint64_t>();
    HORA_TRY(launch_dist_tile(h->metric, TILE_ARGMIN, p, s));
    gk_pick_kernel<<<ceil_div(n, 256), 256, 0, s>>>(keys.as<uint64_t>(), n, labels.as<uint32_t>(), nullptr);
    HORA_LAUNCHED();
    HORA_TRY(sort_labels(nullptr, labels.as<uint32_t>(), n, (int)K, blk, cnt, off.as<int64_t>(),
                         members.as<uint32_t>(), s));
    HORA_TRY(launch_center_sum(X, ld, members.as<uint32_t>(), off.as<int64_t>(), (int)K, dim, 0, NAN,
                               means.as<float>(), s));
  }
  // per mean, the nearest row (the means as queries, exact FP32)
  if (cos) HORA_TRY(launch_row_norms(means.as<float>(), K, ld, dim, cnorm.as<float>(), nullptr, s));
  int retries = 0;
  HORA_TRY(bf_topk_exact(base_view(h), h->metric, means.as<float>(), cnorm.as<float>(), K, 1, h->cand_cap,
                         h->ws, best.as<uint64_t>(), s, &retries));
  gk_pick_kernel<<<ceil_div(K, 256), 256, 0, s>>>(best.as<uint64_t>(), K, nullptr, d_rows.as<uint64_t>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaMemcpyAsync(roots_out, d_rows.ptr, sizeof(uint64_t) * K, cudaMemcpyDeviceToHost, s));
  if (means_out)
    HORA_CUDA_TRY(cudaMemcpy2DAsync(means_out, dim * 4, means.ptr, ld * 4, dim * 4, K, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  return HORA_OK;
}

}  // extern "C"
