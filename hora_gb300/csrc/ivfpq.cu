// ivfpq.cu — IVFPQIndex ("PQIVFIndex") build and search on the GPU.
//
// Build (IVFPQIndex::train, src/index/pq_idx.rs:357-396):
//   coarse k-means over the (training) items with the index metric
//   (Kmeans::train, src/core/kmeans.rs:195-207): init_center, then per epoch
//   assign (exact FP32 tile kernel, strict '<' = smallest (d,row) key),
//   update (centroid sums in FP64 or FP32 in item order, empty -> zero) and
//   split_center (seeded splitmix64 stream, one thread: the reference's
//   walk is sequential);  assign every item -> inverted lists in item order;
//   per (list, subspace) PQ k-means on the residuals x - c_list with 2^bits
//   centres and Euclidean distance (PQIndex::train_center, pq_idx.rs:122-149),
//   one CTA per instance running all epochs;  encode (pq_idx.rs:143-144).
// Search (IVFPQIndex::search_knn_adc, pq_idx.rs:408-439):
//   coarse distances (exact FP32 tile kernel) -> the nprobe nearest lists;
//   (query, list) pairs sorted by list so consecutive CTAs reuse the list's
//   codebook from L1/L2; per pair the LUT (pq_idx.rs:170-179) in shared
//   memory, the ADC scan (pq_idx.rs:182-188, sequential f32 sum over
//   subspaces) and a radix select of the pair's k best; a final per-query
//   merge keeps the k smallest (distance,row) keys.  Optional exact FP32
//   rerank of a widened ADC shortlist (not in the reference; off by default).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "dist_tile.cuh"
#include "index.h"
#include "select.cuh"

namespace hora {

struct IvfState {
  int64_t n_list = 0, n_sub = 0, K = 0, dmax = 0, sub_bits = 0, n_items = 0;
  std::vector<int> sub_begin, sub_len;
  DevBuf sub_begin_d, sub_len_d;
  DevBuf centers;  // n_list x ld (zero padded)
  DevBuf cnorm;    // n_list f32 (cosine)
  DevBuf offsets;  // n_list + 1 int64
  DevBuf items;    // n u32 rows, list order
  DevBuf codes;    // n x n_sub u8, list order
  DevBuf books;    // n_list x n_sub x K x dmax f32
  DevBuf trained;  // n_list u8
  std::vector<int64_t> h_offsets;
  std::vector<uint8_t> h_trained;
  int64_t max_list = 0;
  // every subspace spans 4 dimensions starting at a multiple of 4 (the ADC
  // LUT build then reads each residual slice as one aligned 16-byte load)
  bool sub_aligned4 = false;
  // metric of the PQ stages: Euclidean inside an IVF-PQ index (pq_idx.rs:71),
  // the build metric for a flat PQIndex (pq_idx.rs:198-202)
  int pq_metric = M_L2;
};

void ivf_state_free(IvfState *p) { delete p; }

// The probability walk of Kmeans::split_center (kmeans.rs:150-193) for one
// empty centre, evaluated by one warp 32 candidates at a time.  The
// sequential walk visits centres start, start+1, ... (mod C); a centre with
// a non-zero count takes the next draw u (53 bits) of the splitmix64 stream
// and is picked when u / 2^53 < count / batch, tested exactly as
// u * batch < count * 2^53.  Draw number t uses state s + t * kRngStep, so
// lane l computes its own draw from the number of non-zero centres before
// it in the window; the pick and the stream position after it are those of
// the sequential walk.  All 32 lanes call it; returns -1 after max_windows.
template <typename CountT>
__device__ int split_pick_warp(const CountT *counts, int C, int start, uint64_t batch,
                               uint64_t &s, int64_t max_windows) {
  const int lane = threadIdx.x & 31;
  int base = start;
  for (int64_t w = 0; w < max_windows; ++w) {
    const int cand = (base + lane) % C;
    const uint64_t cnt = (uint64_t)counts[cand];
    const bool nz = cnt > 0;
    const unsigned nzb = __ballot_sync(0xffffffffu, nz);
    bool acc = false;
    if (nz) {
      const unsigned before = __popc(nzb & ((1u << lane) - 1u));
      const uint64_t u = mix64(s + (uint64_t)(before + 1) * kRngStep) >> 11;
      const uint64_t lo = u * batch, hi = __umul64hi(u, batch);
      const uint64_t rhi = cnt >> 11, rlo = cnt << 53;
      acc = hi < rhi || (hi == rhi && lo < rlo);
    }
    const unsigned ab = __ballot_sync(0xffffffffu, acc);
    if (ab) {
      const int first = __ffs(ab) - 1;
      s += (uint64_t)__popc(nzb & (0xffffffffu >> (31 - first))) * kRngStep;
      return (base + first) % C;
    }
    s += (uint64_t)__popc(nzb) * kRngStep;
    base = (base + 32) % C;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// k-means pieces (coarse, full dimension)

// Kmeans::init_center (kmeans.rs:50-86): column means accumulated in item
// order, then mean +1 / -1 with the reference's (i & (1 << j)) == 1 test.
__global__ void coarse_init_kernel(const float *X, int64_t ld, int64_t n, int64_t dim,
                                   int64_t n_center, int accum_f64, float *centers) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= dim) return;
  float mean;
  if (accum_f64) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += (double)X[i * ld + j];
    mean = (float)(s / (double)n);
  } else {
    float s = 0.0f;
    for (int64_t i = 0; i < n; ++i) s = __fadd_rn(s, X[i * ld + j]);
    mean = __fdiv_rn(s, (float)n);
  }
  for (int64_t i = 0; i < n_center; ++i) {
    bool plus = ((uint64_t)i & ((uint64_t)1 << ((uint64_t)j & 63))) == 1;
    centers[i * ld + j] = plus ? __fadd_rn(mean, 1.0f) : __fsub_rn(mean, 1.0f);
  }
}

// Stable counting sort of n labels in [0, C): block histograms, per-label
// block prefix, then an in-order warp scatter inside each block.  An item
// whose label is outside [0, C) (an empty key) is left out of every bucket.
constexpr int kSortBlock = 1024;

__global__ void label_hist_kernel(const uint64_t *keys, const uint32_t *labels, int64_t n, int C, int bs,
                                  uint32_t *block_counts) {
  extern __shared__ uint32_t hist[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) hist[c] = 0;
  __syncthreads();
  int64_t lo = (int64_t)blockIdx.x * bs;
  for (int64_t i = lo + threadIdx.x; i < min(n, lo + bs); i += blockDim.x) {
    uint32_t l = keys ? key_row(keys[i]) : labels[i];
    if (l < (uint32_t)C) atomicAdd(&hist[l], 1u);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) block_counts[(int64_t)blockIdx.x * C + c] = hist[c];
}

// per label: running offsets over blocks; totals -> counts[c].  One warp
// per label, 32 blocks per step (a warp scan of their counts).
__global__ void label_block_scan_kernel(uint32_t *block_counts, int64_t nblocks, int C,
                                        int64_t *counts) {
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= C) return;
  uint32_t run = 0;
  for (int64_t b0 = 0; b0 < nblocks; b0 += 32) {
    const int64_t b = b0 + lane;
    const uint32_t v = b < nblocks ? block_counts[b * C + c] : 0u;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (b < nblocks) block_counts[b * C + c] = run + inc - v;
    run += __shfl_sync(0xffffffffu, inc, 31);
  }
  if (lane == 0) counts[c] = run;
}

// exclusive scan of C counts into offsets[0..C] (one CTA)
__global__ void offsets_scan_kernel(const int64_t *counts, int C, int64_t *offsets) {
  __shared__ int64_t wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = (int)(blockDim.x >> 5);
  const int per = (C + blockDim.x - 1) / blockDim.x;
  const int lo = t * per, hi = min(C, lo + per);
  int64_t s = 0;
  for (int c = lo; c < hi; ++c) s += counts[c];
  // block scan of the threads' sums: within each warp, then over the warps
  int64_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int64_t x = lane < nw ? wsum[lane] : 0;
    int64_t xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane < nw) wsum[lane] = xi - x;
  }
  __syncthreads();
  int64_t run = wsum[w] + inc - s;
  for (int c = lo; c < hi; ++c) {
    offsets[c] = run;
    run += counts[c];
  }
  if (t == (int)blockDim.x - 1) offsets[C] = run;
}

__global__ void label_scatter_kernel(const uint64_t *keys, const uint32_t *labels, int64_t n, int C, int bs,
                                     const uint32_t *block_counts, const int64_t *offsets,
                                     uint32_t *members) {
  extern __shared__ uint32_t rank[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) rank[c] = 0;
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  int64_t lo = (int64_t)blockIdx.x * bs;
  int64_t hi = min(n, lo + bs);
  for (int64_t base = lo; base < hi; base += 32) {
    int64_t i = base + lane;
    uint32_t l = i < hi ? (keys ? key_row(keys[i]) : labels[i]) : 0xffffffffu;
    const bool ok = l < (uint32_t)C;
    unsigned peers = __match_any_sync(0xffffffffu, l);
    unsigned lower = peers & ((1u << lane) - 1u);
    uint32_t r0 = ok ? rank[l] : 0;
    __syncwarp();
    if (ok) {
      uint32_t pos = r0 + __popc(lower);
      members[offsets[l] + block_counts[(int64_t)blockIdx.x * C + l] + pos] = (uint32_t)i;
      if (lower == 0) rank[l] = r0 + __popc(peers);
    }
    __syncwarp();
  }
}

// new centres: per (centre, column) sequential sum over members in item
// order; the loads run 8 members ahead of the (order-preserving) adds
__global__ void center_sum_kernel(const float *X, int64_t ld, const uint32_t *members,
                                  const int64_t *offsets, int C, int64_t dim, int accum_f64,
                                  float empty, float *centers) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)C * dim) return;
  int c = (int)(t / dim);
  int64_t j = t % dim;
  int64_t lo = offsets[c], hi = offsets[c + 1];
  float out = empty;
  if (hi > lo) {
    float v[8];
    if (accum_f64) {
      double s = 0.0;
      int64_t p = lo;
      for (; p + 8 <= hi; p += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = X[(int64_t)members[p + u] * ld + j];
#pragma unroll
        for (int u = 0; u < 8; ++u) s += (double)v[u];
      }
      for (; p < hi; ++p) s += (double)X[(int64_t)members[p] * ld + j];
      out = (float)(s / (double)(hi - lo));
    } else {
      float s = 0.0f;
      int64_t p = lo;
      for (; p + 8 <= hi; p += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = X[(int64_t)members[p + u] * ld + j];
#pragma unroll
        for (int u = 0; u < 8; ++u) s = __fadd_rn(s, v[u]);
      }
      for (; p < hi; ++p) s = __fadd_rn(s, X[(int64_t)members[p] * ld + j]);
      out = __fdiv_rn(s, (float)(hi - lo));
    }
  }
  centers[(int64_t)c * ld + j] = out;
}

int launch_center_sum(const float *X, int64_t ld, const uint32_t *members, const int64_t *offsets,
                      int C, int64_t dim, int accum_f64, float empty, float *centers, cudaStream_t s) {
  center_sum_kernel<<<ceil_div((int64_t)C * dim, 256), 256, 0, s>>>(X, ld, members, offsets, C, dim,
                                                                    accum_f64, empty, centers);
  HORA_LAUNCHED();
  return HORA_OK;
}

// Kmeans::split_center (kmeans.rs:150-193): the empty centres in index
// order, each picking its source with split_pick_warp.  One warp; the walk
// is bounded, status 1 = gave up.
__global__ void split_kernel(float *centers, int64_t ld, int64_t dim, int64_t *counts, int C,
                             int64_t batch, uint64_t *rng_state, int *status) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  const int lane = threadIdx.x;
  uint64_t s = *rng_state;
  const float lo = 1.0f - 1.0f / 1024.0f, hi = 1.0f + 1.0f / 1024.0f;
  for (int i = 0; i < C; ++i) {
    if (counts[i] != 0) continue;  // uniform: every lane reads the same count
    const int sc = split_pick_warp(counts, C, (i + 1) % C, (uint64_t)batch, s, (int64_t)1 << 21);
    if (sc < 0) {
      if (lane == 0) {
        *status = 1;
        *rng_state = s;
      }
      return;
    }
    for (int64_t j = lane; j < dim; j += 32) {
      float v = centers[(int64_t)sc * ld + j];
      if (j % 2 == 0) {
        centers[(int64_t)i * ld + j] = __fmul_rn(v, lo);
        centers[(int64_t)sc * ld + j] = __fmul_rn(v, hi);
      } else {
        centers[(int64_t)i * ld + j] = __fmul_rn(v, hi);
        centers[(int64_t)sc * ld + j] = __fmul_rn(v, lo);
      }
    }
    __syncwarp();
    if (lane == 0) {
      const int64_t half = counts[sc] / 2;
      counts[i] = half;
      counts[sc] -= half;
    }
    __syncwarp();
  }
  if (lane == 0) *rng_state = s;
}

// ---------------------------------------------------------------------------
// PQ: residual sub-vectors, per-instance k-means, encode

// Z[m][p][t] = x[row_p][b_m + t] - c_list[b_m + t]  (kmeans.rs:37-41 order)
__global__ void residual_gather_kernel(const float *X, int64_t ld, const float *centers,
                                       const uint32_t *rows, const uint32_t *row_list,
                                       int64_t npos, int M, int dmax, const int *sb,
                                       const int *sl, float *Z) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npos * M) return;
  int m = (int)(t % M);
  int64_t p = t / M;
  int64_t r = rows[p];
  int64_t c = row_list[p];
  float *z = Z + ((int64_t)m * npos + p) * dmax;
  for (int u = 0; u < dmax; ++u)
    z[u] = u < sl[m] ? __fsub_rn(X[r * ld + sb[m] + u], centers[c * ld + sb[m] + u]) : 0.0f;
}

// metric(z, c) over a DM-wide sub-vector in dimension order (the padding
// beyond the subspace's length is zero on both sides and adds exact zeros)
template <int MT, int DM>
__device__ __forceinline__ float sub_dist(const float *a, const float *b) {
  float s = 0.0f;
#pragma unroll
  for (int u = 0; u < DM; ++u) s = dist_op<MT>(s, a[u], b[u]);
  return s;
}

// Kmeans::search_data's argmin (kmeans.rs:127-148): strict '<' from centre 0
template <int MT, int DM>
__device__ __forceinline__ int sub_argmin(const float *z, const float *cent, int K) {
  int best = 0;
  float bd = sub_dist<MT, DM>(z, cent);
  for (int j = 1; j < K; ++j) {
    const float d = sub_dist<MT, DM>(z, cent + j * DM);
    if (d < bd) {
      bd = d;
      best = j;
    }
  }
  return best;
}

template <int DM>
__device__ __forceinline__ int sub_argmin_mt(int mt, const float *z, const float *cent, int K) {
  return mt == M_L1 ? sub_argmin<M_L1, DM>(z, cent, K)
                    : mt == M_IP ? sub_argmin<M_IP, DM>(z, cent, K) : sub_argmin<M_L2, DM>(z, cent, K);
}

// One CTA per (list, subspace) instance: Kmeans::train on the list's
// residual sub-vectors (PQIndex::train_center, pq_idx.rs:125-146).
template <int DM>
__global__ void __launch_bounds__(256) pq_kmeans_kernel(
    const float *Z, int64_t npos, const int64_t *toff, int M, int K, const int *sl, int epochs,
    uint64_t seed, int accum_f64, int mt, uint8_t *asg_g, uint32_t *mem_g, float *books,
    uint8_t *trained, int *status) {
  extern __shared__ __align__(16) float sm[];
  float *cent = sm;                                  // K x DM
  int64_t *cnt = reinterpret_cast<int64_t *>(cent + K * DM + (K * DM) % 2);  // K
  int *ccount = reinterpret_cast<int *>(cnt + K);    // K members per centre
  int *cstart = ccount + K;                          // K first member slot
  int *ccur = cstart + K;                            // K scatter cursor
  __shared__ float mean[DM];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = blockIdx.x / M, m = blockIdx.x % M;
  const int64_t lo = toff[c], n = toff[c + 1] - lo;
  const int len = sl[m];
  float *book = books + ((int64_t)c * M + m) * K * DM;
  if (n == 0) {
    for (int i = threadIdx.x; i < K * DM; i += blockDim.x) book[i] = 0.0f;
    if (threadIdx.x == 0 && m == 0) trained[c] = 0;
    return;
  }
  const float *z = Z + ((int64_t)m * npos + lo) * DM;
  uint8_t *asg = asg_g + (int64_t)m * npos + lo;
  uint32_t *members = mem_g + (int64_t)m * npos + lo;
  // init_center
  if (threadIdx.x < DM) {
    int u = threadIdx.x;
    float mu = 0.0f;
    if (u < len) {
      if (accum_f64) {
        double s = 0.0;
        for (int64_t i = 0; i < n; ++i) s += (double)z[i * DM + u];
        mu = (float)(s / (double)n);
      } else {
        float s = 0.0f;
        for (int64_t i = 0; i < n; ++i) s = __fadd_rn(s, z[i * DM + u]);
        mu = __fdiv_rn(s, (float)n);
      }
    }
    mean[u] = mu;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < K * DM; e += blockDim.x) {
    int j = e / DM, u = e % DM;
    bool plus = ((uint64_t)j & ((uint64_t)1 << ((uint64_t)u & 63))) == 1;
    cent[e] = u < len ? (plus ? __fadd_rn(mean[u], 1.0f) : __fsub_rn(mean[u], 1.0f)) : 0.0f;
  }
  __syncthreads();
  uint64_t rng = instance_seed(seed, 1 + (uint64_t)c * M + m);
  for (int ep = 0; ep < epochs; ++ep) {
    // search_data: strict '<' from centre 0
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      float zi[DM];
#pragma unroll
      for (int u = 0; u < DM; ++u) zi[u] = z[i * DM + u];
      asg[i] = (uint8_t)sub_argmin_mt<DM>(mt, zi, cent, K);
    }
    __syncthreads();
    // update_center: per centre, members in item order.  The members are
    // bucketed by centre first (a stable counting sort), so each centre's
    // thread reads only its own members.
    for (int j = threadIdx.x; j < K; j += blockDim.x) ccount[j] = 0;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&ccount[asg[i]], 1);
    __syncthreads();
    if (warp == 0) {
      // exclusive scan of the counts (lane l owns centres l*per .. l*per+per-1)
      const int per = (K + 31) / 32;
      int run = 0;
      for (int t = 0; t < per; ++t) {
        const int j = lane * per + t;
        run += j < K ? ccount[j] : 0;
      }
      int inc = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      int at = inc - run;
      for (int t = 0; t < per; ++t) {
        const int j = lane * per + t;
        if (j < K) {
          cstart[j] = at;
          ccur[j] = at;
          at += ccount[j];
        }
      }
      __syncwarp();
      // stable scatter in item order, 32 items at a time
      for (int64_t i0 = 0; i0 < n; i0 += 32) {
        const int64_t i = i0 + lane;
        const bool live = i < n;
        const unsigned act = __ballot_sync(0xffffffffu, live);
        if (live) {
          const int a = asg[i];
          const unsigned peers = __match_any_sync(act, a);
          const int rank = __popc(peers & ((1u << lane) - 1u));
          const int base = ccur[a];
          members[base + rank] = (uint32_t)i;
          __syncwarp(act);
          if (rank == 0) ccur[a] = base + __popc(peers);
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < K; j += blockDim.x) {
      const int b = cstart[j], cn = ccount[j];
      float out[DM];
      if (accum_f64) {
        double s[DM];
#pragma unroll
        for (int u = 0; u < DM; ++u) s[u] = 0.0;
        for (int p = b; p < b + cn; ++p) {
          const float *zr = z + (int64_t)members[p] * DM;
#pragma unroll
          for (int u = 0; u < DM; ++u) s[u] += (double)zr[u];
        }
#pragma unroll
        for (int u = 0; u < DM; ++u) out[u] = cn ? (float)(s[u] / (double)cn) : 0.0f;
      } else {
        float s[DM];
#pragma unroll
        for (int u = 0; u < DM; ++u) s[u] = 0.0f;
        for (int p = b; p < b + cn; ++p) {
          const float *zr = z + (int64_t)members[p] * DM;
#pragma unroll
          for (int u = 0; u < DM; ++u) s[u] = __fadd_rn(s[u], zr[u]);
        }
#pragma unroll
        for (int u = 0; u < DM; ++u) out[u] = cn ? __fdiv_rn(s[u], (float)cn) : 0.0f;
      }
      cnt[j] = cn;
      // no thread reads the centres during the update, so write in place
#pragma unroll
      for (int u = 0; u < DM; ++u) cent[j * DM + u] = out[u];
    }
    __syncthreads();
    if (ep < epochs - 1 && threadIdx.x < 32) {
      // split_center by warp 0 (split_pick_warp); lane 0 owns the counts
      const float lo_ = 1.0f - 1.0f / 1024.0f, hi_ = 1.0f + 1.0f / 1024.0f;
      for (int i0 = 0; i0 < K; i0 += 32) {
        // empty centres of this window in index order; a split only ever
        // empties the centre being filled, so the set ahead stays valid
        unsigned empty = __ballot_sync(0xffffffffu, i0 + lane < K && cnt[i0 + lane] == 0);
        while (empty) {
          const int i = i0 + __ffs(empty) - 1;
          empty &= empty - 1;
          const int sc = split_pick_warp(cnt, K, (i + 1) % K, (uint64_t)n, rng, (int64_t)1 << 19);
          if (sc < 0) {
            if (lane == 0) atomicExch(status, 1);
            i0 = K;
            break;
          }
          if (lane < len) {
            const int u = lane;
            float v = cent[sc * DM + u];
            if (u % 2 == 0) {
              cent[i * DM + u] = __fmul_rn(v, lo_);
              cent[sc * DM + u] = __fmul_rn(v, hi_);
            } else {
              cent[i * DM + u] = __fmul_rn(v, hi_);
              cent[sc * DM + u] = __fmul_rn(v, lo_);
            }
          }
          __syncwarp();
          if (lane == 0) {
            const int64_t half = cnt[sc] / 2;
            cnt[i] = half;
            cnt[sc] -= half;
          }
          __syncwarp();
        }
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < K * DM; e += blockDim.x) book[e] = cent[e];
  if (threadIdx.x == 0 && m == 0) trained[c] = 1;
}

// codes of every list member (pq_idx.rs:143-144): strict '<' argmin per subspace
template <int DM>
__global__ void __launch_bounds__(256) pq_encode_kernel(
    const float *X, int64_t ld, const float *centers, const uint32_t *items, const int64_t *offs,
    const float *books, int M, int K, const int *sb, const int *sl, int mt, uint8_t *codes) {
  extern __shared__ __align__(16) float cb[];  // K x DM
  const int c = blockIdx.x, m = blockIdx.y;
  const int64_t lo = offs[c], n = offs[c + 1] - lo;
  if (n == 0) return;
  const float *book = books + ((int64_t)c * M + m) * K * DM;
  for (int e = threadIdx.x; e < K * DM; e += blockDim.x) cb[e] = book[e];
  __syncthreads();
  const int b = sb[m], len = sl[m];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    int64_t r = items[lo + i];
    float zi[DM];
#pragma unroll
    for (int u = 0; u < DM; ++u)
      zi[u] = u < len ? __fsub_rn(X[r * ld + b + u], centers[(int64_t)c * ld + b + u]) : 0.0f;
    codes[(lo + i) * M + m] = (uint8_t)sub_argmin_mt<DM>(mt, zi, cb, K);
  }
}

// ---------------------------------------------------------------------------
// search

// Pairs (query, probe slot) grouped by list: histogram / scan / scatter.
__global__ void pair_hist_kernel(const uint64_t *probes, int64_t nq, int pmax, int jbegin,
                                 const uint32_t *nprobe_q, int C, int64_t *cnt) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * pmax) return;
  int64_t q = t / pmax;
  int j = (int)(t % pmax);
  int p = nprobe_q ? (int)nprobe_q[q] : pmax;
  uint64_t k = probes[t];
  if (j < jbegin || j >= p || k == kEmptyKey) return;
  atomicAdd(reinterpret_cast<unsigned long long *>(cnt + key_row(k)), 1ull);
}

// Per query: the number of ADC candidates its probe slots [jbegin, nprobe)
// hold ((nprobe - jbegin) x R, contiguous from slot jbegin), and empty keys
// in any slot of that range whose probe is empty (no pair was formed), so
// the merge reads exactly the slots this call wrote.
__global__ void pair_counts_kernel(const uint64_t *probes, int64_t nq, int pmax, int jbegin,
                                   const uint32_t *nprobe_q, int R, uint64_t *cand, uint32_t *count) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * pmax) return;
  const int64_t q = t / pmax;
  const int j = (int)(t % pmax);
  const int p = nprobe_q ? min((int)nprobe_q[q], pmax) : pmax;
  if (j == 0) count[q] = (uint32_t)(p > jbegin ? (p - jbegin) * R : 0);
  if (j >= jbegin && j < p && probes[t] == kEmptyKey)
    for (int r = 0; r < R; ++r) cand[t * R + r] = kEmptyKey;
}

__global__ void pair_scatter_kernel(const uint64_t *probes, int64_t nq, int pmax, int jbegin,
                                    const uint32_t *nprobe_q, int C, const int64_t *off,
                                    int64_t *cursor, uint32_t *pq, uint32_t *pc, uint32_t *pslot) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * pmax) return;
  int64_t q = t / pmax;
  int j = (int)(t % pmax);
  int p = nprobe_q ? (int)nprobe_q[q] : pmax;
  uint64_t k = probes[t];
  if (j < jbegin || j >= p || k == kEmptyKey) return;
  uint32_t c = key_row(k);
  int64_t pos = off[c] + (int64_t)atomicAdd(reinterpret_cast<unsigned long long *>(cursor + c), 1ull);
  pq[pos] = (uint32_t)q;
  pc[pos] = c;
  pslot[pos] = (uint32_t)j;
}

// Groups of pairs: per list c, ceil(cnt[c] / G) groups of up to G pairs
// (the list's pairs in scatter order).  One CTA computes the exclusive scans
// of the pair counts (pair_off, C + 1 entries) and of the group counts
// (grp_off, C + 1 entries; grp_off[C] = the number of groups).
__global__ void group_scan_kernel(const int64_t *cnt, int C, int G, int64_t *pair_off, int64_t *grp_off) {
  __shared__ int64_t part_p[1024], part_g[1024];
  const int t = threadIdx.x;
  const int per = (C + blockDim.x - 1) / blockDim.x;
  const int lo = t * per, hi = min(C, lo + per);
  int64_t sp = 0, sg = 0;
  for (int c = lo; c < hi; ++c) {
    sp += cnt[c];
    sg += (cnt[c] + G - 1) / G;
  }
  part_p[t] = sp;
  part_g[t] = sg;
  __syncthreads();
  if (t == 0) {
    int64_t rp = 0, rg = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const int64_t vp = part_p[i], vg = part_g[i];
      part_p[i] = rp;
      part_g[i] = rg;
      rp += vp;
      rg += vg;
    }
    pair_off[C] = rp;
    grp_off[C] = rg;
  }
  __syncthreads();
  int64_t rp = part_p[t], rg = part_g[t];
  for (int c = lo; c < hi; ++c) {
    pair_off[c] = rp;
    grp_off[c] = rg;
    rp += cnt[c];
    rg += (cnt[c] + G - 1) / G;
  }
}

constexpr int kAdcThreads = 512;
static_assert(kAdcThreads % 128 == 0, "the code-major LUT build fixes m per thread");
constexpr int kAdcChunk = 2048;  // code rows scored per selection round

// G sums over subspaces of LUT[m][code[m]] (one per query of the group),
// each in subspace order (pq_idx.rs:180-186).  The LUT holds the G queries'
// entries of one (m, j) side by side (one 4G-byte load per code byte); the
// code row is read VB bytes at a time (VB divides M and the row pitch, so
// every load is aligned); KC = K when it is a compile-time 256.
template <int G, int VB, int KC>
__device__ __forceinline__ void adc_row_g(const uint8_t *code, const float *lut, int M, int Kr,
                                          float (&d)[G]) {
  const int K = KC ? KC : Kr;
#pragma unroll
  for (int g = 0; g < G; ++g) d[g] = 0.0f;
  auto add = [&](int m, uint32_t j) {
    const int e = m * K + (int)j;
    if (G == 4) {
      const float4 v = reinterpret_cast<const float4 *>(lut)[e];
      d[0] = __fadd_rn(d[0], v.x);
      d[1 % G] = __fadd_rn(d[1 % G], v.y);
      d[2 % G] = __fadd_rn(d[2 % G], v.z);
      d[3 % G] = __fadd_rn(d[3 % G], v.w);
    } else if (G == 2) {
      const float2 v = reinterpret_cast<const float2 *>(lut)[e];
      d[0] = __fadd_rn(d[0], v.x);
      d[1 % G] = __fadd_rn(d[1 % G], v.y);
    } else {
      d[0] = __fadd_rn(d[0], lut[e]);
    }
  };
  if (VB == 16) {
    const uint4 *p = reinterpret_cast<const uint4 *>(code);
    for (int gq = 0; gq < M / 16; ++gq) {
      const uint4 w = __ldg(p + gq);
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const uint32_t wt = t < 4 ? w.x : t < 8 ? w.y : t < 12 ? w.z : w.w;
        add(gq * 16 + t, (wt >> (8 * (t & 3))) & 255u);
      }
    }
  } else if (VB == 8) {
    const uint2 *p = reinterpret_cast<const uint2 *>(code);
    for (int gq = 0; gq < M / 8; ++gq) {
      const uint2 w = __ldg(p + gq);
#pragma unroll
      for (int t = 0; t < 8; ++t) add(gq * 8 + t, ((t < 4 ? w.x : w.y) >> (8 * (t & 3))) & 255u);
    }
  } else if (VB == 4) {
    const uint32_t *p = reinterpret_cast<const uint32_t *>(code);
    for (int gq = 0; gq < M / 4; ++gq) {
      const uint32_t w = __ldg(p + gq);
#pragma unroll
      for (int t = 0; t < 4; ++t) add(gq * 4 + t, (w >> (8 * t)) & 255u);
    }
  } else {
    for (int m = 0; m < M; ++m) add(m, __ldg(code + m));
  }
}

// The same sums for a 32-subspace code row already in registers (two
// 16-byte words), K = 256, from a LUT laid out code-major (entry (m, j) at
// j * 32 + m: for 16-byte entries the bank group is m mod 8).  Lane l
// starts its row sk = l mod 8 steps late: at step s it adds subspace s - sk,
// so the eight lanes of a quarter warp read eight different m, one bank
// group each, and every 16-byte gather is conflict-free; each lane still adds
// its subspaces in order 0..31 (bit-identical sums).  The code row is
// shifted by sk bytes once, so that step s reads byte s of it.
// Two f32 additions / subtractions in one instruction (sm_100 and later),
// each lane rounded to nearest-even as __fadd_rn / __fsub_rn round it: the
// same bits as the two scalar operations.
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
  float2 r;
  asm("{ .reg .b64 x, y, z; mov.b64 x, {%2, %3}; mov.b64 y, {%4, %5}; add.rn.f32x2 z, x, y; mov.b64 {%0, %1}, z; }"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
  float2 r;
  asm("{ .reg .b64 x, y, z; mov.b64 x, {%2, %3}; mov.b64 y, {%4, %5}; sub.rn.f32x2 z, x, y; mov.b64 {%0, %1}, z; }"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
// The products stay scalar: with a packed multiply feeding a packed add,
// distances came out one rounding away from the scalar sequence's (the pair
// was fused), while a scalar multiply with an explicit rounding is never
// fused.
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
  return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}

template <int G>
__device__ __forceinline__ void adc_row32_skew_g(const uint4 w0, const uint4 w1, const float *lut, int sk,
                                                 float (&d)[G]) {
#pragma unroll
  for (int g = 0; g < G; ++g) d[g] = 0.0f;
  float2 d01 = make_float2(0.0f, 0.0f), d23 = d01;  // G = 4: two queries per packed add
  const uint32_t c[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
  // B = the 32 code bytes moved up by sk bytes (10 words, zero filled)
  const int q = sk >> 2, r = 8 * (sk & 3);
  uint32_t B[10];
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t a0 = i - 1 >= 0 && i - 1 < 8 ? c[i - 1] : 0u, a1 = i < 8 ? c[i] : 0u;
    const uint32_t b0 = i - 2 >= 0 && i - 2 < 8 ? c[i - 2] : 0u;
    const uint32_t s0 = __funnelshift_l(a0, a1, r);  // q = 0: (c[i] << r) | (c[i-1] >> (32 - r))
    const uint32_t s1 = __funnelshift_l(b0, a0, r);  // q = 1: one word further up
    B[i] = q ? s1 : s0;
  }
#pragma unroll
  for (int st = 0; st < 39; ++st) {
    const int m = st - sk;
    if ((unsigned)m < 32u) {
      const int j = (int)((B[st >> 2] >> (8 * (st & 3))) & 255u);
      const int e = j * 32 + m;
      if (G == 4) {
        const float4 v = reinterpret_cast<const float4 *>(lut)[e];
        d01 = add2_rn(d01, make_float2(v.x, v.y));
        d23 = add2_rn(d23, make_float2(v.z, v.w));
      } else if (G == 2) {
        const float2 v = reinterpret_cast<const float2 *>(lut)[e];
        d[0] = __fadd_rn(d[0], v.x);
        d[1 % G] = __fadd_rn(d[1 % G], v.y);
      } else {
        d[0] = __fadd_rn(d[0], lut[e]);
      }
    }
  }
  if (G == 4) {
    d[0] = d01.x;
    d[1 % G] = d01.y;
    d[2 % G] = d23.x;
    d[3 % G] = d23.y;
  }
}

// LUT[m][j] for the G queries of a group from one load of the codeword
// C[m][j] (pq_idx.rs:170-179: metric(z[range_m], C[m][j]) summed in t order;
// Euclidean inside IVF-PQ, the build metric for a flat PQIndex).  With
// 4-float codewords (DMC = 4) every thread has 8 codeword loads in flight
// before it computes; other widths read the codeword per query.
template <int G, int MT>
__device__ __forceinline__ void lut_store_g(float *lut, int e, const float (&acc)[G]) {
  if (G == 4)
    reinterpret_cast<float4 *>(lut)[e] = make_float4(acc[0], acc[1 % G], acc[2 % G], acc[3 % G]);
  else if (G == 2)
    reinterpret_cast<float2 *>(lut)[e] = make_float2(acc[0], acc[1 % G]);
  else
    lut[e] = acc[0];
}

template <int G, int MT, int DMC>
__device__ __forceinline__ void lut_build_g(const float *book, const float *zq, int dz, const int *sbs,
                                            const int *sls, int M, int K, int kbits, int dm, bool tr,
                                            float *lut) {
  // work item i computes entry (m, j) into LUT slot m K + j (m-major), or
  // with tr (M = 32, K = 256) into slot j 32 + m (code-major); then the 32
  // items of a warp cover 8 consecutive m x 4 consecutive j, so its codeword
  // loads are 8 runs of 64 bytes and each quarter warp stores 8 consecutive
  // slots (conflict-free)
  const int MK = M * K;
  auto entry_of = [&](int i, int &m, int &j, int &slot) {
    if (tr) {
      m = (i & 7) | (((i >> 5) & 3) << 3);
      j = ((i >> 3) & 3) | ((i >> 7) << 2);
      slot = j * 32 + m;
    } else {
      m = i >> kbits;
      j = i & (K - 1);
      slot = i;
    }
  };
  if (DMC == 4 && tr) {
    // every subspace spans 4 dimensions starting at a multiple of 4, and with
    // the code-major mapping (blockDim a multiple of 128) a thread's items all
    // share one m: its queries' residual slices are loaded once
    const float4 *b4 = reinterpret_cast<const float4 *>(book);
    const int m = (threadIdx.x & 7) | (((threadIdx.x >> 5) & 3) << 3);
    float4 z[G];
#pragma unroll
    for (int g = 0; g < G; ++g) z[g] = *reinterpret_cast<const float4 *>(zq + g * dz + sbs[m]);
    for (int i0 = threadIdx.x; i0 < MK; i0 += 8 * blockDim.x) {
      float4 cv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < MK) cv[u] = __ldg(b4 + m * K + (((i >> 3) & 3) | ((i >> 7) << 2)));
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < MK) {
          float acc[G];
          if (MT == M_L2 && G == 4) {
            // two queries per packed sub / mul / add, each query's sum in
            // the order and rounding of dist_op
            float2 a01 = make_float2(0.0f, 0.0f), a23 = a01;
            const float cd[4] = {cv[u].x, cv[u].y, cv[u].z, cv[u].w};
            const float z0[4] = {z[0].x, z[0].y, z[0].z, z[0].w}, z1[4] = {z[1 % G].x, z[1 % G].y, z[1 % G].z, z[1 % G].w};
            const float z2[4] = {z[2 % G].x, z[2 % G].y, z[2 % G].z, z[2 % G].w};
            const float z3[4] = {z[3 % G].x, z[3 % G].y, z[3 % G].z, z[3 % G].w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const float2 c2 = make_float2(cd[t], cd[t]);
              const float2 t01 = sub2_rn(make_float2(z0[t], z1[t]), c2);
              const float2 t23 = sub2_rn(make_float2(z2[t], z3[t]), c2);
              a01 = add2_rn(a01, mul2_rn(t01, t01));
              a23 = add2_rn(a23, mul2_rn(t23, t23));
            }
            acc[0] = a01.x;
            acc[1 % G] = a01.y;
            acc[2 % G] = a23.x;
            acc[3 % G] = a23.y;
          } else {
#pragma unroll
            for (int g = 0; g < G; ++g) {
              float a = dist_op<MT>(0.0f, z[g].x, cv[u].x);
              a = dist_op<MT>(a, z[g].y, cv[u].y);
              a = dist_op<MT>(a, z[g].z, cv[u].z);
              acc[g] = dist_op<MT>(a, z[g].w, cv[u].w);
            }
          }
          lut_store_g<G, MT>(lut, (((i >> 3) & 3) | ((i >> 7) << 2)) * 32 + m, acc);
        }
      }
    }
  } else if (DMC == 4) {
    // every subspace spans 4 dimensions starting at a multiple of 4: the
    // residual slice of each query is one aligned 16-byte load
    const float4 *b4 = reinterpret_cast<const float4 *>(book);
    for (int i0 = threadIdx.x; i0 < MK; i0 += 8 * blockDim.x) {
      float4 cv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < MK) {
          int m, j, slot;
          entry_of(i, m, j, slot);
          cv[u] = __ldg(b4 + m * K + j);
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i < MK) {
          int m, j, slot;
          entry_of(i, m, j, slot);
          const int zo = sbs[m];
          float acc[G];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const float4 z = *reinterpret_cast<const float4 *>(zq + g * dz + zo);
            float a = dist_op<MT>(0.0f, z.x, cv[u].x);
            a = dist_op<MT>(a, z.y, cv[u].y);
            a = dist_op<MT>(a, z.z, cv[u].z);
            acc[g] = dist_op<MT>(a, z.w, cv[u].w);
          }
          lut_store_g<G, MT>(lut, slot, acc);
        }
      }
    }
  } else {
    for (int i = threadIdx.x; i < MK; i += blockDim.x) {
      int m, j, slot;
      entry_of(i, m, j, slot);
      const int len = sls[m];
      const float *cj = book + (int64_t)(m * K + j) * dm;
      float acc[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const float *z = zq + g * dz + sbs[m];
        float a = 0.0f;
        for (int t = 0; t < len; ++t) a = dist_op<MT>(a, z[t], __ldg(cj + t));
        acc[g] = a;
      }
      lut_store_g<G, MT>(lut, slot, acc);
    }
  }
}

// Per list of a group, the selection state (ints): the range of the
// distance words, the radix digit position, keys still to take, prefix and
// mask of the digits fixed so far, done, phase (0: distance digits, 1: row
// digits among the keys equal to tau, 2: the keys of the k-th key's bin
// ranked in one warp), tau, the row bound, the compaction count, the keys
// of that bin gathered for the rank.
enum : int {
  kStMin = 0, kStMax, kStShift, kStRem, kStPrefix, kStMask, kStDone, kStPhase, kStTau, kStRBound,
  kStCnt, kStBCnt, kStWords = 16
};
constexpr int kSelDigitBits = 11, kSelNB = 1 << kSelDigitBits;
// A bin holding the k-th key and at most this many keys in all is settled
// by ranking its keys instead of another radix pass over the list.
constexpr int kSelRankMax = 32;

// Every lane of the warp: the bin of a kSelNB-bin histogram whose
// cumulative count first reaches rem (1 <= rem <= total) and the count below
// it.  Lane l owns bins [nb l, nb l + nb), nb = kSelNB / 32, summed in a
// rotated order (conflict-free banks); the warp then scans the chosen lane's
// nb bins together, two per lane.
__device__ __forceinline__ void warp_find_bin_all(const uint32_t *hist, uint32_t rem, int &bin,
                                                  uint32_t &below) {
  constexpr int nb = kSelNB / 32;
  const int lane = threadIdx.x & 31;
  uint32_t sum = 0;
#pragma unroll 16
  for (int i = 0; i < nb; ++i) sum += hist[lane * nb + ((i + lane) & (nb - 1))];
  uint32_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const uint32_t exc = inc - sum;
  const unsigned who = __ballot_sync(0xffffffffu, exc < rem && inc >= rem);
  const int src = who ? __ffs(who) - 1 : 31;
  const uint32_t base = __shfl_sync(0xffffffffu, exc, src);
  // the chosen lane's nb bins: bins 2 l, 2 l + 1 of its range on lane l
  static_assert(nb % 2 == 0 && nb <= 64, "two bins per lane");
  const uint32_t b0 = 2 * lane < nb ? hist[src * nb + 2 * lane] : 0u;
  const uint32_t b1 = 2 * lane + 1 < nb ? hist[src * nb + 2 * lane + 1] : 0u;
  uint32_t pinc = b0 + b1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, pinc, o);
    if (lane >= o) pinc += y;
  }
  const uint32_t pexc = base + pinc - (b0 + b1);
  const bool first = pexc < rem && pexc + b0 >= rem;
  const bool second = !first && pexc + b0 < rem && pexc + b0 + b1 >= rem;
  const unsigned w2 = __ballot_sync(0xffffffffu, first || second);
  const int l2 = w2 ? __ffs(w2) - 1 : 31;
  const int d = src * nb + 2 * lane + (second ? 1 : 0);
  const uint32_t run = second ? pexc + b0 : pexc;
  bin = __shfl_sync(0xffffffffu, w2 ? d : src * nb + nb - 1, l2);
  below = __shfl_sync(0xffffffffu, run, l2);
}

// The CTA keeps, for each of the gc lists of a group, the k smallest keys
// (distance word, row) of its L = held + ch entries: distance words dk[g *
// stride + i], rows hrow[g * k + i] for i < held (the kept head) and
// crow[i - held] after it (the chunk, shared by the lists); rows are
// distinct within a list, so the selection is exact.  A radix select for
// all lists at once (every thread works in every pass): 11-bit digits of
// the distance word minus the list's minimum, from the top of its range,
// stopping per list once the k-th key's bin is taken whole, or once that
// bin holds at most kSelRankMax keys: the compaction then gathers them
// (bd / brow, kSelRankMax words per list) and one warp ranks them by
// (distance, row), which saves the further passes over the whole list; a
// list whose k-th distance is tied past the last digit in a larger bin
// continues on the row digits of the tied keys.  The kept keys go through
// od / orow to the head.  st holds the per-list state (kStWords ints per
// list, kStMin / kStMax already set by the caller); hist is zero on entry
// and on return.  0 < k < L.
template <int G>
__device__ __forceinline__ void cta_select_group(uint32_t *dk, int stride, uint32_t *hrow,
                                                 const uint32_t *crow, int held, int gc, int L, int k,
                                                 uint32_t *hist, int *st, uint32_t *od, uint32_t *orow,
                                                 uint32_t *bd, uint32_t *brow) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < gc) {
    int *q = st + threadIdx.x * kStWords;
    const uint32_t span = (uint32_t)q[kStMax] - (uint32_t)q[kStMin];
    const int sh = 32 - __clz((int)span) - kSelDigitBits;  // __clz(0) = 32
    q[kStShift] = sh < 0 ? 0 : sh;
    q[kStRem] = k;
    q[kStPrefix] = 0;
    q[kStMask] = 0;
    q[kStDone] = 0;
    q[kStPhase] = 0;
    q[kStTau] = 0;
    q[kStRBound] = -1;
    q[kStCnt] = 0;
    q[kStBCnt] = 0;
  }
  __syncthreads();
  for (int pass = 0; pass < 2 * (32 + kSelDigitBits - 1) / kSelDigitBits; ++pass) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g >= gc) break;
      const int *q = st + g * kStWords;
      if (q[kStDone]) continue;
      const uint32_t prefix = (uint32_t)q[kStPrefix], mask = (uint32_t)q[kStMask];
      const int shift = q[kStShift];
      uint32_t *h = hist + g * kSelNB;
      if (q[kStPhase] == 0) {
        const uint32_t kmin = (uint32_t)q[kStMin];
        for (int i = threadIdx.x; i < L; i += blockDim.x) {
          const uint32_t d = dk[g * stride + i] - kmin;
          if ((d & mask) == prefix) atomicAdd(&h[(d >> shift) & (kSelNB - 1)], 1u);
        }
      } else {
        const uint32_t tau = (uint32_t)q[kStTau];
        for (int i = threadIdx.x; i < L; i += blockDim.x) {
          if (dk[g * stride + i] != tau) continue;
          const uint32_t r = i < held ? hrow[g * k + i] : crow[i - held];
          if ((r & mask) == prefix) atomicAdd(&h[(r >> shift) & (kSelNB - 1)], 1u);
        }
      }
    }
    __syncthreads();
    if (warp < gc && !st[warp * kStWords + kStDone]) {
      int *q = st + warp * kStWords;
      uint32_t *h = hist + warp * kSelNB;
      int bin;
      uint32_t below;
      warp_find_bin_all(h, (uint32_t)q[kStRem], bin, below);
      const uint32_t at = h[bin];
      __syncwarp();
      for (int i = lane; i < kSelNB; i += 32) h[i] = 0;
      if (lane == 0) {
        const int shift = q[kStShift];
        const uint32_t rem = (uint32_t)q[kStRem] - below;
        const uint32_t prefix = (uint32_t)q[kStPrefix] | ((uint32_t)bin << shift);
        const uint32_t low = shift ? (1u << shift) - 1u : 0u;
        q[kStRem] = (int)rem;
        if (at == rem) {  // every key of this bin is kept
          if (q[kStPhase] == 0) {
            q[kStTau] = (int)((uint32_t)q[kStMin] + (prefix | low));
            q[kStRBound] = -1;
          } else {
            q[kStRBound] = (int)(prefix | low);
          }
          q[kStDone] = 1;
        } else if (q[kStPhase] == 0 && at <= (uint32_t)kSelRankMax) {
          // few keys share the bin: the compaction gathers them and one
          // warp takes the rem smallest (distance, row) among them
          q[kStPrefix] = (int)prefix;
          q[kStMask] = (int)((uint32_t)q[kStMask] | ((uint32_t)(kSelNB - 1) << shift));
          q[kStPhase] = 2;
          q[kStDone] = 1;
        } else if (shift == 0 && q[kStPhase] == 0) {
          // the k-th distance itself, tied: the smallest rows among the ties
          q[kStTau] = (int)((uint32_t)q[kStMin] + prefix);
          q[kStPhase] = 1;
          q[kStShift] = 32 - kSelDigitBits;
          q[kStPrefix] = 0;
          q[kStMask] = 0;
        } else if (shift == 0) {  // unreachable with distinct rows
          q[kStRBound] = (int)prefix;
          q[kStDone] = 1;
        } else {
          q[kStPrefix] = (int)prefix;
          q[kStMask] = (int)((uint32_t)q[kStMask] | ((uint32_t)(kSelNB - 1) << shift));
          q[kStShift] = shift > kSelDigitBits ? shift - kSelDigitBits : 0;
        }
      }
    }
    __syncthreads();
    bool all = true;
    for (int g = 0; g < gc; ++g) all = all && st[g * kStWords + kStDone];
    if (all) break;
  }
  // kept: distance below tau, or equal with the row at or below the bound;
  // a list in phase 2 keeps the keys below its bin and gathers the bin's
#pragma unroll
  for (int g = 0; g < G; ++g) {
    if (g >= gc) break;
    int *cnt = st + g * kStWords + kStCnt;
    if (st[g * kStWords + kStPhase] == 2) {
      const uint32_t kmin = (uint32_t)st[g * kStWords + kStMin];
      const uint32_t prefix = (uint32_t)st[g * kStWords + kStPrefix], mask = (uint32_t)st[g * kStWords + kStMask];
      int *bcnt = st + g * kStWords + kStBCnt;
      for (int i = threadIdx.x; i < L; i += blockDim.x) {
        const uint32_t d = dk[g * stride + i], dd = d - kmin;
        if (dd < prefix) {
          const int pos = atomicAdd(cnt, 1);
          if (pos < k) {
            od[g * k + pos] = d;
            orow[g * k + pos] = i < held ? hrow[g * k + i] : crow[i - held];
          }
        } else if ((dd & mask) == prefix) {
          const int b = atomicAdd(bcnt, 1);
          if (b < kSelRankMax) {
            bd[g * kSelRankMax + b] = d;
            brow[g * kSelRankMax + b] = i < held ? hrow[g * k + i] : crow[i - held];
          }
        }
      }
      continue;
    }
    const uint32_t tau = (uint32_t)st[g * kStWords + kStTau], rb = (uint32_t)st[g * kStWords + kStRBound];
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      const uint32_t d = dk[g * stride + i];
      if (d > tau) continue;
      const uint32_t r = i < held ? hrow[g * k + i] : crow[i - held];
      if (d < tau || r <= rb) {
        const int pos = atomicAdd(cnt, 1);
        if (pos < k) {
          od[g * k + pos] = d;
          orow[g * k + pos] = r;
        }
      }
    }
  }
  __syncthreads();
  // phase 2: the rank of each gathered key among them by (distance, row);
  // the rem smallest follow the keys below the bin
  if (warp < gc && st[warp * kStWords + kStPhase] == 2) {
    const int *q = st + warp * kStWords;
    const int n = min(q[kStBCnt], kSelRankMax), rem = q[kStRem], base = q[kStCnt];
    const uint32_t d = lane < n ? bd[warp * kSelRankMax + lane] : 0xffffffffu;
    const uint32_t r = lane < n ? brow[warp * kSelRankMax + lane] : 0xffffffffu;
    int rank = 0;
#pragma unroll
    for (int j = 0; j < kSelRankMax; ++j) {
      const uint32_t dj = __shfl_sync(0xffffffffu, d, j), rj = __shfl_sync(0xffffffffu, r, j);
      rank += j < n && (dj < d || (dj == d && rj < r));
    }
    const int pos = base + rank;
    if (lane < n && rank < rem && pos < k) {
      od[warp * k + pos] = d;
      orow[warp * k + pos] = r;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < gc * k; t += blockDim.x) {
    const int g = t / k, r = t - g * k;
    dk[g * stride + r] = od[t];
    hrow[t] = orow[t];
  }
  __syncthreads();
}

// The G-wide LUT's floats, rounded up to a multiple of 4 so that the
// residual queries behind it start on a 16-byte boundary.
__host__ __device__ inline size_t adc_lut_floats(int G, int M, int K) {
  return ((size_t)M * K * G + 3) & ~(size_t)3;
}

// Dynamic shared memory of adc_group_kernel: the G-wide LUT, the G residual
// queries, per query the distance words of the kept R plus a chunk and the
// rows of the kept R, the rows of a chunk, per query a selection histogram,
// 2 R words of selection output and 2 kSelRankMax words of ranked keys, the
// selection state, the subspace table.
__host__ __device__ inline size_t adc_group_smem(int G, int M, int K, int dz, int R) {
  return sizeof(float) * (adc_lut_floats(G, M, K) + (size_t)G * dz) +
         sizeof(uint32_t) * ((size_t)G * (kAdcChunk + R) + (size_t)G * R + kAdcChunk +
                             (size_t)G * kSelNB + (size_t)2 * G * R + (size_t)2 * G * kSelRankMax) +
         sizeof(int) * ((size_t)kStWords * G + 2 * M);
}

// One CTA per group of up to G (query, probe slot) pairs of one list
// (IVFPQIndex::search_knn_adc per probed list, pq_idx.rs:165-194 and
// 424-437): the G residuals z = q - c_list, one LUT build that reads the
// list's codebook once for all G queries, one pass over the list's code
// rows in chunks that reads each row once and scores it for all G queries
// (the ADC sums bit-identical to a per-query scan), and per chunk a radix
// select keeping each query's R smallest (distance, row) keys.  Output: the
// pair's R keys at cand[(q * pmax + slot) * R ...], empty keys past the
// list's length.  The CTAs are persistent: each takes the next group from
// *next (zero before the launch) until grp_off[C] groups are done; gmap
// gives each group's list.
template <int G, int VB>
__global__ void __launch_bounds__(kAdcThreads, 1) adc_group_kernel(
    const float *Q, int64_t ldq, const float *centers, int64_t ldc, const float *books,
    const uint8_t *codes, const uint32_t *items, const int64_t *offs, const uint8_t *trained,
    const uint32_t *pq, const uint32_t *pslot, const int64_t *pair_off, const int64_t *grp_off,
    const uint32_t *gmap, int C, int M, int K, int dm, int aligned4, const int *sb, const int *sl,
    int mt, int R, int pmax, uint64_t *cand, unsigned long long *next) {
  const int64_t T = grp_off[C];
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_c, s_gc;
  __shared__ long long s_p0, s_b;
  const int dcov = sb[M - 1] + sl[M - 1];
  const int dz = (dcov + 3) & ~3;
  const int stride = kAdcChunk + R;
  float *lut = reinterpret_cast<float *>(smraw);                       // M * K * G (rounded to 4)
  float *zq = lut + adc_lut_floats(G, M, K);                           // G * dz, 16-byte aligned
  uint32_t *dk = reinterpret_cast<uint32_t *>(zq + G * dz);           // G * (R + chunk)
  uint32_t *hrow = dk + G * stride;                                    // G * R
  uint32_t *crow = hrow + G * R;                                       // chunk
  uint32_t *hist = crow + kAdcChunk;                                   // G * kSelNB
  uint32_t *od = hist + G * kSelNB;                                    // G * R
  uint32_t *orow = od + G * R;                                         // G * R
  uint32_t *bd = orow + G * R;                                         // G * kSelRankMax
  uint32_t *brow = bd + G * kSelRankMax;                               // G * kSelRankMax
  int *st = reinterpret_cast<int *>(brow + G * kSelRankMax);           // G * kStWords
  int *sbs = st + G * kStWords;                                        // M
  int *sls = sbs + M;                                                  // M
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    sbs[m] = sb[m];
    sls[m] = sl[m];
  }
  for (int t = threadIdx.x; t < G * kSelNB; t += blockDim.x) hist[t] = 0;
  const int kbits = 31 - __clz(K);  // K = 2^sub_bits
  for (;;) {
    if (threadIdx.x == 0) {
      const long long b = (long long)atomicAdd(next, 1ull);
      s_b = b;
      if (b < T) {
        const int c = (int)gmap[b];
        const int64_t p0 = pair_off[c] + (b - grp_off[c]) * G;
        s_c = c;
        s_p0 = p0;
        s_gc = (int)min((int64_t)G, pair_off[c + 1] - p0);
      }
    }
    __syncthreads();
    if (s_b >= T) return;
    const int c = s_c, gc = s_gc;
    const int64_t p0 = s_p0;
    const int64_t lrow = offs[c], L = offs[c + 1] - lrow;
    if (!trained[c] || L == 0) {
      for (int t = threadIdx.x; t < gc * R; t += blockDim.x) {
        const int64_t pi = p0 + t / R;
        cand[((int64_t)pq[pi] * pmax + pslot[pi]) * R + t % R] = kEmptyKey;
      }
      __syncthreads();  // s_c / s_p0 / s_gc are read before the next group overwrites them
      continue;
    }
    // z = q - c_list over the covered dimensions (pq_idx.rs:158-161); group
    // slots past gc repeat the first query (their results are not written)
    for (int t = threadIdx.x; t < G * dcov; t += blockDim.x) {
      const int g = t / dcov, u = t - g * dcov;
      const int64_t q = pq[p0 + (g < gc ? g : 0)];
      zq[g * dz + u] = __fsub_rn(Q[q * ldq + u], centers[(int64_t)c * ldc + u]);
    }
    __syncthreads();
    const float *book = books + (int64_t)c * M * K * dm;
    // 32-byte code rows and 256 centroids: the skewed scan reads a code-major LUT
    const bool tr = VB == 16 && M == 32 && K == 256;
    if (mt == M_L2 && aligned4)
      lut_build_g<G, M_L2, 4>(book, zq, dz, sbs, sls, M, K, kbits, dm, tr, lut);
    else if (mt == M_L2)
      lut_build_g<G, M_L2, 0>(book, zq, dz, sbs, sls, M, K, kbits, dm, tr, lut);
    else if (mt == M_L1)
      lut_build_g<G, M_L1, 0>(book, zq, dz, sbs, sls, M, K, kbits, dm, tr, lut);
    else
      lut_build_g<G, M_IP, 0>(book, zq, dz, sbs, sls, M, K, kbits, dm, tr, lut);
    const uint8_t *lcodes = codes + lrow * M;
    int held = 0;
    for (int64_t c0 = 0; c0 < L; c0 += kAdcChunk) {
      const int ch = (int)min((int64_t)kAdcChunk, L - c0);
      if (threadIdx.x < G) {
        st[threadIdx.x * kStWords + kStMin] = -1;  // 0xffffffff as unsigned
        st[threadIdx.x * kStWords + kStMax] = 0;
      }
      __syncthreads();  // the LUT is built; the previous chunk's selection is done
      uint32_t kmin[G], kmax[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        kmin[g] = 0xffffffffu;
        kmax[g] = 0u;
      }
      for (int i = threadIdx.x; i < held; i += blockDim.x) {  // the kept head is in the range
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const uint32_t v = dk[g * stride + i];
          kmin[g] = min(kmin[g], v);
          kmax[g] = max(kmax[g], v);
        }
      }
      if (VB == 16 && M == 32 && K == 256) {
        // 32-byte code rows: the next row's words are loaded while this
        // row is scored
        const uint4 *rows4 = reinterpret_cast<const uint4 *>(lcodes + c0 * 32);
        int i = threadIdx.x;
        uint4 w0 = make_uint4(0, 0, 0, 0), w1 = w0;
        uint32_t row = 0;
        if (i < ch) {
          w0 = __ldg(rows4 + 2 * i);
          w1 = __ldg(rows4 + 2 * i + 1);
          row = items[lrow + c0 + i];
        }
        for (; i < ch; i += blockDim.x) {
          const int in = i + blockDim.x;
          uint4 n0 = w0, n1 = w1;
          uint32_t nrow = 0;
          if (in < ch) {
            n0 = __ldg(rows4 + 2 * in);
            n1 = __ldg(rows4 + 2 * in + 1);
            nrow = items[lrow + c0 + in];
          }
          float d[G];
          adc_row32_skew_g<G>(w0, w1, lut, threadIdx.x & 7, d);
          crow[i] = row;
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const uint32_t v = f2ord(d[g]);
            dk[g * stride + held + i] = v;
            kmin[g] = min(kmin[g], v);
            kmax[g] = max(kmax[g], v);
          }
          w0 = n0;
          w1 = n1;
          row = nrow;
        }
      } else {
        for (int i = threadIdx.x; i < ch; i += blockDim.x) {
          float d[G];
          if (K == 256)
            adc_row_g<G, VB, 256>(lcodes + (c0 + i) * M, lut, M, K, d);
          else
            adc_row_g<G, VB, 0>(lcodes + (c0 + i) * M, lut, M, K, d);
          crow[i] = items[lrow + c0 + i];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const uint32_t v = f2ord(d[g]);
            dk[g * stride + held + i] = v;
            kmin[g] = min(kmin[g], v);
            kmax[g] = max(kmax[g], v);
          }
        }
      }
      const int tot = held + ch;
      if (tot > R) {
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const uint32_t lo = __reduce_min_sync(0xffffffffu, kmin[g]);
          const uint32_t hi = __reduce_max_sync(0xffffffffu, kmax[g]);
          if ((threadIdx.x & 31) == 0 && g < gc) {
            atomicMin(reinterpret_cast<unsigned *>(&st[g * kStWords + kStMin]), lo);
            atomicMax(reinterpret_cast<unsigned *>(&st[g * kStWords + kStMax]), hi);
          }
        }
        __syncthreads();
        cta_select_group<G>(dk, stride, hrow, crow, held, gc, tot, R, hist, st, od, orow, bd, brow);
        held = R;
      } else {
        // short so far: the chunk's rows join the head as they are
        __syncthreads();
        for (int t = threadIdx.x; t < gc * ch; t += blockDim.x) {
          const int g = t / ch, i = t - g * ch;
          hrow[g * R + held + i] = crow[i];
        }
        held = tot;
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < gc * R; t += blockDim.x) {
      const int g = t / R, r = t - g * R;
      const int64_t pi = p0 + g;
      cand[((int64_t)pq[pi] * pmax + pslot[pi]) * R + r] =
          r < held ? (((uint64_t)dk[g * stride + r] << 32) | hrow[g * R + r]) : kEmptyKey;
    }
    __syncthreads();  // the group's shared state is read before the next group overwrites it
  }
}

// Group g's list: for every list c, the groups grp_off[c] .. grp_off[c+1].
__global__ void group_map_kernel(const int64_t *grp_off, int C, uint32_t *gmap) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  for (int64_t g = grp_off[c]; g < grp_off[c + 1]; ++g) gmap[g] = (uint32_t)c;
}

// ---------------------------------------------------------------------------
// host side

int sort_labels(const uint64_t *keys, const uint32_t *labels, int64_t n, int C,
                       DevBuf &blk, DevBuf &counts, int64_t *d_offsets, uint32_t *d_members,
                       cudaStream_t s) {
  // items per block: kSortBlock, or for small sets (a search's queries)
  // fewer, so that the scatter's serial walk of each block is spread over
  // the SMs; the order (stable by item) is the same either way
  const int bs = n > (int64_t)2 * 152 * kSortBlock ? kSortBlock
                                                   : (int)std::max<int64_t>(128, round_up(ceil_div(n, (int64_t)2 * 152), 32));
  int64_t nb = ceil_div(n, (int64_t)bs);
  HORA_TRY(blk.reserve(sizeof(uint32_t) * nb * C));
  HORA_TRY(counts.reserve(sizeof(int64_t) * C));
  int smem = C * 4;
  HORA_SMEM_ATTR(label_hist_kernel, smem);
  HORA_SMEM_ATTR(label_scatter_kernel, smem);
  {
    ProfScope ps("ivf_sort", s);
    label_hist_kernel<<<(unsigned)nb, 256, smem, s>>>(keys, labels, n, C, bs, blk.as<uint32_t>());
    HORA_LAUNCHED();
    label_block_scan_kernel<<<ceil_div((int64_t)C * 32, 256), 256, 0, s>>>(blk.as<uint32_t>(), nb, C,
                                                                            counts.as<int64_t>());
    HORA_LAUNCHED();
    offsets_scan_kernel<<<1, 1024, 0, s>>>(counts.as<int64_t>(), C, d_offsets);
    HORA_LAUNCHED();
    label_scatter_kernel<<<(unsigned)nb, 256, smem, s>>>(keys, labels, n, C, bs, blk.as<uint32_t>(),
                                                        d_offsets, d_members);
    HORA_LAUNCHED();
  }
  return HORA_OK;
}

static int pq_dmax_of(int64_t dim, int64_t n_sub) {
  int64_t sd = dim / n_sub;
  return (int)(sd + ((dim % sd) ? 1 : 0));
}

static int dm_bucket(int dmax) { return dmax <= 1 ? 1 : dmax <= 2 ? 2 : dmax <= 4 ? 4 : dmax <= 8 ? 8 : 16; }

template <int DM>
static int launch_pq_kmeans(IvfState &v, const float *Z, int64_t npos, const int64_t *toff,
                            int epochs, uint64_t seed, int accum, uint8_t *asg, uint32_t *mem, int *status,
                            cudaStream_t s) {
  int smem = (int)(v.K * DM * 4 + 8 + v.K * 8 + 3 * v.K * 4 + 16);
  HORA_SMEM_ATTR(pq_kmeans_kernel<DM>, smem);
  ProfScope ps("pq_kmeans", s);
  pq_kmeans_kernel<DM><<<(unsigned)(v.n_list * v.n_sub), 256, smem, s>>>(
      Z, npos, toff, (int)v.n_sub, (int)v.K, v.sub_len_d.as<int>(), epochs, seed, accum, v.pq_metric, asg, mem,
      v.books.as<float>(), v.trained.as<uint8_t>(), status);
  HORA_LAUNCHED();
  return HORA_OK;
}

template <int DM>
static int launch_pq_encode(IvfState &v, const float *X, int64_t ld, cudaStream_t s) {
  int smem = (int)(v.K * DM * 4);
  dim3 grid((unsigned)v.n_list, (unsigned)v.n_sub);
  ProfScope ps("pq_encode", s);
  pq_encode_kernel<DM><<<grid, 256, smem, s>>>(X, ld, v.centers.as<float>(), v.items.as<uint32_t>(),
                                               v.offsets.as<int64_t>(), v.books.as<float>(),
                                               (int)v.n_sub, (int)v.K, v.sub_begin_d.as<int>(),
                                               v.sub_len_d.as<int>(), v.pq_metric, v.codes.as<uint8_t>());
  HORA_LAUNCHED();
  return HORA_OK;
}

static int encode_all(hora_index *h, IvfState &v, cudaStream_t s) {
  const float *X = h->base.as<float>();
  switch (dm_bucket((int)v.dmax)) {
    case 1: return launch_pq_encode<1>(v, X, h->ld, s);
    case 2: return launch_pq_encode<2>(v, X, h->ld, s);
    case 4: return launch_pq_encode<4>(v, X, h->ld, s);
    case 8: return launch_pq_encode<8>(v, X, h->ld, s);
    default: return launch_pq_encode<16>(v, X, h->ld, s);
  }
}

static void init_layout(hora_index *h, IvfState &v) {
  v.pq_metric = h->kind == HORA_INDEX_PQ ? h->metric : M_L2;
  v.n_list = (int64_t)h->ivf.n_kmeans_center;
  v.n_sub = (int64_t)h->ivf.n_sub;
  v.sub_bits = (int64_t)h->ivf.sub_bits;
  v.K = (int64_t)1 << v.sub_bits;
  v.dmax = dm_bucket(pq_dmax_of((int64_t)h->dim, v.n_sub));
  // PQIndex::new subspace ranges (pq_idx.rs:75-88), dimension % sub_dimension as written
  int64_t sd = (int64_t)h->dim / v.n_sub, r = (int64_t)h->dim % sd;
  v.sub_begin.resize(v.n_sub);
  v.sub_len.resize(v.n_sub);
  for (int64_t i = 0; i < v.n_sub; ++i) {
    int64_t b, e;
    if (i < r) {
      b = i * (sd + 1);
      e = (i + 1) * (sd + 1);
    } else {
      b = r * (sd + 1) + (i - r) * sd;
      e = r * (sd + 1) + (i + 1 - r) * sd;
    }
    v.sub_begin[i] = (int)b;
    v.sub_len[i] = (int)(e - b);
  }
  v.sub_aligned4 = v.dmax == 4;
  for (int64_t i = 0; i < v.n_sub; ++i)
    v.sub_aligned4 = v.sub_aligned4 && v.sub_begin[i] == 4 * i && v.sub_len[i] == 4;
}

static int upload_layout(IvfState &v, cudaStream_t s) {
  HORA_TRY(v.sub_begin_d.reserve(sizeof(int) * v.n_sub));
  HORA_TRY(v.sub_len_d.reserve(sizeof(int) * v.n_sub));
  HORA_CUDA_TRY(cudaMemcpyAsync(v.sub_begin_d.ptr, v.sub_begin.data(), sizeof(int) * v.n_sub,
                                cudaMemcpyHostToDevice, s));
  HORA_CUDA_TRY(cudaMemcpyAsync(v.sub_len_d.ptr, v.sub_len.data(), sizeof(int) * v.n_sub,
                                cudaMemcpyHostToDevice, s));
  return HORA_OK;
}

// Assigns every item to its nearest centre (index metric) and builds the
// inverted lists in item order.
static int assign_lists(hora_index *h, IvfState &v, DevBuf &keys, DevBuf &blk, DevBuf &cnt,
                        cudaStream_t s) {
  const int64_t n = h->n;
  HORA_TRY(keys.reserve(sizeof(uint64_t) * n));
  if (h->metric == M_COS) {
    HORA_TRY(v.cnorm.reserve(sizeof(float) * v.n_list));
    HORA_TRY(launch_row_norms(v.centers.as<float>(), v.n_list, h->ld, h->dim, v.cnorm.as<float>(), nullptr, s));
    HORA_TRY(ensure_norms(h, s));
  }
  TileParams p;
  p.Q = h->base.as<float>();
  p.ldq = h->ld;
  p.nq = n;
  p.X = v.centers.as<float>();
  p.ldx = h->ld;
  p.r_begin = 0;
  p.r_end = v.n_list;
  p.ld = h->ld;
  p.qnorm = h->xnorm.as<float>();
  p.xnorm = v.cnorm.as<float>();
  p.out_key = keys.as<uint64_t>();
  HORA_TRY(launch_dist_tile(h->metric, TILE_ARGMIN, p, s));
  HORA_TRY(v.offsets.reserve(sizeof(int64_t) * (v.n_list + 1)));
  HORA_TRY(v.items.reserve(sizeof(uint32_t) * std::max<int64_t>(n, 1)));
  HORA_TRY(sort_labels(keys.as<uint64_t>(), nullptr, n, (int)v.n_list, blk, cnt,
                       v.offsets.as<int64_t>(), v.items.as<uint32_t>(), s));
  return HORA_OK;
}

static int fetch_offsets(IvfState &v, cudaStream_t s) {
  v.h_offsets.resize(v.n_list + 1);
  HORA_CUDA_TRY(cudaMemcpyAsync(v.h_offsets.data(), v.offsets.ptr, sizeof(int64_t) * (v.n_list + 1),
                                cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  v.max_list = 0;
  for (int64_t c = 0; c < v.n_list; ++c) v.max_list = std::max(v.max_list, v.h_offsets[c + 1] - v.h_offsets[c]);
  return HORA_OK;
}

int ivf_build(hora_index *h) {
  cudaStream_t s = h->stream;
  if (h->n == 0) return fail(HORA_EINVAL, "None to assigned impossible split center");
  std::unique_ptr<IvfState, IvfDeleter> vp(new IvfState());
  IvfState &v = *vp;
  init_layout(h, v);
  if (v.n_list > h->n) {
    // more centres than items is legal in the reference; lists simply stay empty
  }
  HORA_TRY(upload_layout(v, s));
  const int64_t n = h->n;
  const int64_t T = (h->train_size > 0 && (int64_t)h->train_size < n) ? (int64_t)h->train_size : n;
  const int C = (int)v.n_list;
  const int epochs = (int)h->ivf.train_epoch;
  const float *X = h->base.as<float>();
  HORA_TRY(v.centers.reserve(sizeof(float) * C * h->ld));
  HORA_CUDA_TRY(cudaMemsetAsync(v.centers.ptr, 0, sizeof(float) * C * h->ld, s));
  DevBuf keys, blk, cnt, members, moff, state;
  HORA_TRY(state.reserve(64));
  HORA_CUDA_TRY(cudaMemsetAsync(state.ptr, 0, 64, s));
  uint64_t seed0 = instance_seed(h->seed, 0);
  HORA_CUDA_TRY(cudaMemcpyAsync(state.ptr, &seed0, 8, cudaMemcpyHostToDevice, s));
  uint64_t *d_rng = state.as<uint64_t>();
  int *d_status = reinterpret_cast<int *>(state.as<char>() + 8);

  // ---- coarse k-means on the first T items (a flat PQIndex has one list
  //      centred at zero: no coarse stage, residual = the vector itself) ----
  const bool flat = h->kind == HORA_INDEX_PQ;
  if (!flat) {
    ProfScope ps("coarse_init", s);
    coarse_init_kernel<<<ceil_div(h->dim, 128), 128, 0, s>>>(X, h->ld, T, h->dim, C, h->accum_f64,
                                                             v.centers.as<float>());
    HORA_LAUNCHED();
  }
  HORA_TRY(keys.reserve(sizeof(uint64_t) * T));
  HORA_TRY(members.reserve(sizeof(uint32_t) * T));
  HORA_TRY(moff.reserve(sizeof(int64_t) * (C + 1)));
  if (h->metric == M_COS) {
    HORA_TRY(ensure_norms(h, s));
    HORA_TRY(v.cnorm.reserve(sizeof(float) * C));
  }
  for (int ep = 0; ep < (flat ? 0 : epochs); ++ep) {
    if (h->metric == M_COS)
      HORA_TRY(launch_row_norms(v.centers.as<float>(), C, h->ld, h->dim, v.cnorm.as<float>(), nullptr, s));
    TileParams p;
    p.Q = X;
    p.ldq = h->ld;
    p.nq = T;
    p.X = v.centers.as<float>();
    p.ldx = h->ld;
    p.r_begin = 0;
    p.r_end = C;
    p.ld = h->ld;
    p.qnorm = h->xnorm.as<float>();
    p.xnorm = v.cnorm.as<float>();
    p.out_key = keys.as<uint64_t>();
    HORA_TRY(launch_dist_tile(h->metric, TILE_ARGMIN, p, s));
    HORA_TRY(sort_labels(keys.as<uint64_t>(), nullptr, T, C, blk, cnt, moff.as<int64_t>(),
                         members.as<uint32_t>(), s));
    {
      ProfScope ps("coarse_update", s);
      HORA_TRY(launch_center_sum(X, h->ld, members.as<uint32_t>(), moff.as<int64_t>(), C, h->dim,
                                 h->accum_f64, 0.0f, v.centers.as<float>(), s));
    }
    if (ep < epochs - 1) {
      ProfScope ps("coarse_split", s);
      split_kernel<<<1, 32, 0, s>>>(v.centers.as<float>(), h->ld, h->dim, cnt.as<int64_t>(), C, T,
                                   d_rng, d_status);
      HORA_LAUNCHED();
    }
  }
  // ---- inverted lists over every item ----
  HORA_TRY(assign_lists(h, v, keys, blk, cnt, s));
  HORA_TRY(fetch_offsets(v, s));
  v.n_items = n;

  // ---- training rows per list: members among the first T items (all
  //      members when a list has none of them) ----
  std::vector<uint32_t> h_items(n);
  HORA_CUDA_TRY(cudaMemcpyAsync(h_items.data(), v.items.ptr, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int64_t> toff(C + 1, 0);
  std::vector<uint32_t> trows, tlist;
  trows.reserve(T);
  tlist.reserve(T);
  for (int c = 0; c < C; ++c) {
    int64_t lo = v.h_offsets[c], hi = v.h_offsets[c + 1];
    int64_t nt = 0;
    for (int64_t p = lo; p < hi; ++p) nt += h_items[p] < (uint64_t)T;
    for (int64_t p = lo; p < hi; ++p)
      if (nt == 0 || h_items[p] < (uint64_t)T) {
        trows.push_back(h_items[p]);
        tlist.push_back((uint32_t)c);
      }
    toff[c + 1] = (int64_t)trows.size();
  }
  const int64_t npos = (int64_t)trows.size();
  DevBuf d_toff, d_trows, d_tlist, Z, asg, mem;
  HORA_TRY(d_toff.reserve(sizeof(int64_t) * (C + 1)));
  HORA_TRY(d_trows.reserve(sizeof(uint32_t) * std::max<int64_t>(npos, 1)));
  HORA_TRY(d_tlist.reserve(sizeof(uint32_t) * std::max<int64_t>(npos, 1)));
  HORA_TRY(Z.reserve(sizeof(float) * std::max<int64_t>(npos, 1) * v.n_sub * v.dmax));
  HORA_TRY(asg.reserve(std::max<int64_t>(npos, 1) * v.n_sub));
  HORA_TRY(mem.reserve(sizeof(uint32_t) * std::max<int64_t>(npos, 1) * v.n_sub));
  HORA_CUDA_TRY(cudaMemcpyAsync(d_toff.ptr, toff.data(), sizeof(int64_t) * (C + 1), cudaMemcpyHostToDevice, s));
  if (npos) {
    HORA_CUDA_TRY(cudaMemcpyAsync(d_trows.ptr, trows.data(), sizeof(uint32_t) * npos, cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(d_tlist.ptr, tlist.data(), sizeof(uint32_t) * npos, cudaMemcpyHostToDevice, s));
    ProfScope ps("pq_residuals", s);
    residual_gather_kernel<<<ceil_div(npos * v.n_sub, 256), 256, 0, s>>>(
        X, h->ld, v.centers.as<float>(), d_trows.as<uint32_t>(), d_tlist.as<uint32_t>(), npos,
        (int)v.n_sub, (int)v.dmax, v.sub_begin_d.as<int>(), v.sub_len_d.as<int>(), Z.as<float>());
    HORA_LAUNCHED();
  }
  HORA_TRY(v.books.reserve(sizeof(float) * C * v.n_sub * v.K * v.dmax));
  HORA_TRY(v.trained.reserve(C));
  HORA_CUDA_TRY(cudaMemsetAsync(v.trained.ptr, 0, C, s));
  switch (v.dmax) {
    case 1: HORA_TRY(launch_pq_kmeans<1>(v, Z.as<float>(), npos, d_toff.as<int64_t>(), epochs, h->seed, h->accum_f64, asg.as<uint8_t>(), mem.as<uint32_t>(), d_status, s)); break;
    case 2: HORA_TRY(launch_pq_kmeans<2>(v, Z.as<float>(), npos, d_toff.as<int64_t>(), epochs, h->seed, h->accum_f64, asg.as<uint8_t>(), mem.as<uint32_t>(), d_status, s)); break;
    case 4: HORA_TRY(launch_pq_kmeans<4>(v, Z.as<float>(), npos, d_toff.as<int64_t>(), epochs, h->seed, h->accum_f64, asg.as<uint8_t>(), mem.as<uint32_t>(), d_status, s)); break;
    case 8: HORA_TRY(launch_pq_kmeans<8>(v, Z.as<float>(), npos, d_toff.as<int64_t>(), epochs, h->seed, h->accum_f64, asg.as<uint8_t>(), mem.as<uint32_t>(), d_status, s)); break;
    default: HORA_TRY(launch_pq_kmeans<16>(v, Z.as<float>(), npos, d_toff.as<int64_t>(), epochs, h->seed, h->accum_f64, asg.as<uint8_t>(), mem.as<uint32_t>(), d_status, s)); break;
  }
  // ---- codes of every member ----
  HORA_TRY(v.codes.reserve(std::max<int64_t>(n, 1) * v.n_sub));
  HORA_TRY(encode_all(h, v, s));
  int status = 0;
  HORA_CUDA_TRY(cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  v.h_trained.resize(C);
  HORA_CUDA_TRY(cudaMemcpyAsync(v.h_trained.data(), v.trained.ptr, C, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  if (status) return fail(HORA_ETIMEDOUT, "k-means split walk did not terminate");
  if (h->metric == M_COS) {
    HORA_TRY(v.cnorm.reserve(sizeof(float) * C));
    HORA_TRY(launch_row_norms(v.centers.as<float>(), C, h->ld, h->dim, v.cnorm.as<float>(), nullptr, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  h->ivfs = std::move(vp);
  h->coarse_tc.reset();  // the centres' image follows the centres
  return HORA_OK;
}

int ivf_set_codebooks(hora_index *h, const float *centers, const float *codebooks) {
  cudaStream_t s = h->stream;
  if (h->n == 0) return fail(HORA_EINVAL, "no items");
  if (h->metric == M_UNKNOWN) return fail(HORA_EMETRIC, "unknown method: build first or set a metric");
  std::unique_ptr<IvfState, IvfDeleter> vp(new IvfState());
  IvfState &v = *vp;
  init_layout(h, v);
  HORA_TRY(upload_layout(v, s));
  const int C = (int)v.n_list;
  HORA_TRY(v.centers.reserve(sizeof(float) * C * h->ld));
  HORA_CUDA_TRY(cudaMemsetAsync(v.centers.ptr, 0, sizeof(float) * C * h->ld, s));
  HORA_CUDA_TRY(cudaMemcpy2DAsync(v.centers.ptr, h->ld * 4, centers, h->dim * 4, h->dim * 4, C,
                                  cudaMemcpyDefault, s));
  // host codebooks are [C][M][K][dmax_exact]; device keeps dmax bucket
  const int dexact = pq_dmax_of((int64_t)h->dim, v.n_sub);
  HORA_TRY(v.books.reserve(sizeof(float) * C * v.n_sub * v.K * v.dmax));
  HORA_CUDA_TRY(cudaMemsetAsync(v.books.ptr, 0, sizeof(float) * C * v.n_sub * v.K * v.dmax, s));
  HORA_CUDA_TRY(cudaMemcpy2DAsync(v.books.ptr, v.dmax * 4, codebooks, dexact * 4, dexact * 4,
                                  (size_t)C * v.n_sub * v.K, cudaMemcpyDefault, s));
  DevBuf keys, blk, cnt;
  HORA_TRY(assign_lists(h, v, keys, blk, cnt, s));
  HORA_TRY(fetch_offsets(v, s));
  v.n_items = h->n;
  HORA_TRY(v.trained.reserve(C));
  v.h_trained.assign(C, 0);
  for (int c = 0; c < C; ++c) v.h_trained[c] = v.h_offsets[c + 1] > v.h_offsets[c];
  HORA_CUDA_TRY(cudaMemcpyAsync(v.trained.ptr, v.h_trained.data(), C, cudaMemcpyHostToDevice, s));
  HORA_TRY(v.codes.reserve(std::max<int64_t>(h->n, 1) * v.n_sub));
  HORA_TRY(encode_all(h, v, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  h->ivfs = std::move(vp);
  h->coarse_tc.reset();  // the centres' image follows the centres
  h->built = true;
  return HORA_OK;
}

template <int G, int VB>
static int launch_adc_g(IvfState &v, SearchWorkspace &ws, const float *Q, int64_t ldq, int64_t ldc,
                        int64_t max_groups, int dz, int R, int pmax, uint64_t *cand, cudaStream_t s) {
  const size_t smem = adc_group_smem(G, (int)v.n_sub, (int)v.K, dz, R);
  HORA_SMEM_ATTR((adc_group_kernel<G, VB>), smem);
  if (max_groups <= 0) return HORA_OK;
  // persistent CTAs: as many as are resident at once, at most one per group
  int dev = 0, nsm = 0, per_sm = 0;
  HORA_CUDA_TRY(cudaGetDevice(&dev));
  HORA_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  HORA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adc_group_kernel<G, VB>, kAdcThreads, smem));
  const int64_t grid = std::min<int64_t>(max_groups, (int64_t)nsm * std::max(per_sm, 1));
  HORA_TRY(ws.adc_next.reserve(sizeof(unsigned long long)));
  HORA_CUDA_TRY(cudaMemsetAsync(ws.adc_next.ptr, 0, sizeof(unsigned long long), s));
  ProfScope ps("adc_scan", s);
  adc_group_kernel<G, VB><<<(unsigned)grid, kAdcThreads, smem, s>>>(
      Q, ldq, v.centers.as<float>(), ldc, v.books.as<float>(), v.codes.as<uint8_t>(),
      v.items.as<uint32_t>(), v.offsets.as<int64_t>(), v.trained.as<uint8_t>(), ws.pair_q.as<uint32_t>(),
      ws.pair_slot.as<uint32_t>(), ws.pair_off.as<int64_t>(), ws.pair_off.as<int64_t>() + (v.n_list + 1),
      ws.adc_gmap.as<uint32_t>(), (int)v.n_list, (int)v.n_sub, (int)v.K, (int)v.dmax, v.sub_aligned4 ? 1 : 0,
      v.sub_begin_d.as<int>(), v.sub_len_d.as<int>(), v.pq_metric, R, pmax, cand,
      ws.adc_next.as<unsigned long long>());
  HORA_LAUNCHED();
  return HORA_OK;
}

// Code rows are n_sub bytes apart: the widest load that divides n_sub.
template <int G>
static int launch_adc_vb(IvfState &v, SearchWorkspace &ws, const float *Q, int64_t ldq, int64_t ldc,
                         int64_t max_groups, int dz, int R, int pmax, uint64_t *cand, cudaStream_t s) {
  if (v.n_sub % 16 == 0) return launch_adc_g<G, 16>(v, ws, Q, ldq, ldc, max_groups, dz, R, pmax, cand, s);
  if (v.n_sub % 8 == 0) return launch_adc_g<G, 8>(v, ws, Q, ldq, ldc, max_groups, dz, R, pmax, cand, s);
  if (v.n_sub % 4 == 0) return launch_adc_g<G, 4>(v, ws, Q, ldq, ldc, max_groups, dz, R, pmax, cand, s);
  return launch_adc_g<G, 1>(v, ws, Q, ldq, ldc, max_groups, dz, R, pmax, cand, s);
}

// Queries per ADC group: the most (4, 2 or 1) whose shared memory fits.
constexpr size_t kAdcSmemMax = 227 * 1024;  // dynamic shared memory a CTA may use

static int adc_group_width(const IvfState &v, int dz, int R) {
  for (int G = 4; G > 1; G >>= 1)
    if (adc_group_smem(G, (int)v.n_sub, (int)v.K, dz, R) <= kAdcSmemMax) return G;
  return 1;
}

int ivf_pmax(const hora_index *h, int64_t nprobe) {
  const int64_t C = (int64_t)h->ivf.n_kmeans_center;
  int64_t pmax = nprobe > 0 ? nprobe : (int64_t)h->ivf.search_n_center;
  if (pmax > C) pmax = C;  // the reference pops an empty heap (panics) here
  if (pmax < 1) pmax = 1;
  return (int)pmax;
}

// Coarse distances of the staged queries to every centre and each query's
// pmax nearest lists, ascending (pq_idx.rs:416-425).
int ivf_probe(hora_index *h, int64_t nq, int pmax, SearchWorkspace &ws, cudaStream_t s) {
  IvfState &v = *h->ivfs;
  const int C = (int)v.n_list;
  HORA_TRY(ws.coarse.reserve(sizeof(float) * nq * C));
  if (coarse_tc_eligible(h)) {
    // the same probes from a BF16 pass and a certified exact rescoring
    HORA_TRY(ws.probes.reserve(sizeof(uint64_t) * nq * pmax));
    return coarse_tc_probe(h, v.centers.as<float>(), v.cnorm.as<float>(), C, nq, pmax, ws, ws.coarse.as<float>(),
                           ws.probes.as<uint64_t>(), s);
  }
  TileParams p;
  p.Q = ws.q.as<float>();
  p.ldq = h->ld;
  p.nq = nq;
  p.X = v.centers.as<float>();
  p.ldx = h->ld;
  p.r_begin = 0;
  p.r_end = C;
  p.ld = h->ld;
  p.qnorm = ws.qnorm.as<float>();
  p.xnorm = v.cnorm.as<float>();
  p.out_dist = ws.coarse.as<float>();
  p.ldo = C;
  HORA_TRY(launch_dist_tile(h->metric, TILE_DIST, p, s));
  HORA_TRY(ws.probes.reserve(sizeof(uint64_t) * nq * pmax));
  HORA_TRY(launch_rows_topk(ws.coarse.as<float>(), nq, C, C, pmax, ws.probes.as<uint64_t>(), s));
  return HORA_OK;
}

const uint64_t *ivf_probe_keys(const SearchWorkspace &ws) { return ws.probes.as<uint64_t>(); }

// ADC over the probe slots [jbegin, min(nprobe_q, pmax)) of every query,
// merged into M (nq x R keys, kept sorted; the caller initialises it).
int ivf_adc_merge(hora_index *h, int64_t nq, int pmax, int jbegin, const uint32_t *d_nprobe,
                  int R, uint64_t *M, SearchWorkspace &ws, cudaStream_t s) {
  IvfState &v = *h->ivfs;
  const int C = (int)v.n_list;
  const float *Q = ws.q.as<float>();
  const int dcov = v.sub_begin.back() + v.sub_len.back();
  const int dz = (dcov + 3) & ~3;
  const int G = adc_group_width(v, dz, R);
  if (adc_group_smem(G, (int)v.n_sub, (int)v.K, dz, R) > kAdcSmemMax)
    return fail(HORA_ECAP, "IVF-PQ: LUT too large for shared memory");
  HORA_TRY(ws.pair_cnt.reserve(sizeof(int64_t) * (C + 1) * 2));
  HORA_TRY(ws.pair_off.reserve(sizeof(int64_t) * (C + 1) * 2));  // pair offsets, then group offsets
  int64_t *cnt = ws.pair_cnt.as<int64_t>();
  int64_t *cursor = cnt + (C + 1);
  int64_t *poff = ws.pair_off.as<int64_t>();
  HORA_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (C + 1) * 2, s));
  const int64_t tot = nq * pmax;
  // pairs (query, probe slot) grouped by list, no host round trip: the ADC
  // grid is an upper bound on the number of groups
  const int64_t max_pairs = nq * (int64_t)(pmax - jbegin);
  if (max_pairs <= 0) return HORA_OK;
  const int64_t max_groups = ceil_div(max_pairs, G) + std::min<int64_t>(C, max_pairs);
  HORA_TRY(ws.adc_gmap.reserve(sizeof(uint32_t) * max_groups));
  HORA_TRY(ws.pair_q.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  HORA_TRY(ws.pair_c.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  HORA_TRY(ws.pair_slot.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  {
    ProfScope ps("ivf_pairs", s);
    pair_hist_kernel<<<ceil_div(tot, 256), 256, 0, s>>>(ws.probes.as<uint64_t>(), nq, pmax, jbegin,
                                                       d_nprobe, C, cnt);
    HORA_LAUNCHED();
    group_scan_kernel<<<1, 1024, 0, s>>>(cnt, C, G, poff, poff + (C + 1));
    HORA_LAUNCHED();
    group_map_kernel<<<ceil_div(C, 256), 256, 0, s>>>(poff + (C + 1), C, ws.adc_gmap.as<uint32_t>());
    HORA_LAUNCHED();
    pair_scatter_kernel<<<ceil_div(tot, 256), 256, 0, s>>>(
        ws.probes.as<uint64_t>(), nq, pmax, jbegin, d_nprobe, C, poff, cursor,
        ws.pair_q.as<uint32_t>(), ws.pair_c.as<uint32_t>(), ws.pair_slot.as<uint32_t>());
    HORA_LAUNCHED();
  }
  // LUT + ADC scan + per-pair R best; the merge reads only the slots written
  // (the grouped merge for very wide rerank lists reads every slot)
  const int width = pmax * R;
  const bool grouped = !(R <= 256 || merge_smem_bytes(R, width) <= 200 * 1024);
  HORA_TRY(ws.ivf_cand.reserve(sizeof(uint64_t) * nq * pmax * R));
  if (grouped) HORA_CUDA_TRY(cudaMemsetAsync(ws.ivf_cand.ptr, 0xff, sizeof(uint64_t) * nq * pmax * R, s));
  HORA_TRY(ws.count.reserve(sizeof(uint32_t) * std::max<int64_t>(nq, 1)));
  {
    ProfScope ps("ivf_pairs", s);
    pair_counts_kernel<<<ceil_div(tot, 256), 256, 0, s>>>(ws.probes.as<uint64_t>(), nq, pmax, jbegin,
                                                         d_nprobe, R, ws.ivf_cand.as<uint64_t>(),
                                                         ws.count.as<uint32_t>());
    HORA_LAUNCHED();
  }
  uint64_t *cand = ws.ivf_cand.as<uint64_t>();
  switch (G) {
    case 4: HORA_TRY(launch_adc_vb<4>(v, ws, Q, h->ld, h->ld, max_groups, dz, R, pmax, cand, s)); break;
    case 2: HORA_TRY(launch_adc_vb<2>(v, ws, Q, h->ld, h->ld, max_groups, dz, R, pmax, cand, s)); break;
    default: HORA_TRY(launch_adc_vb<1>(v, ws, Q, h->ld, h->ld, max_groups, dz, R, pmax, cand, s)); break;
  }
  // per-query merge of the candidates (pq_idx.rs:429-436): each query's
  // slots [jbegin, nprobe) are contiguous, so the merge reads
  // count[q] = (nprobe - jbegin) x R keys from slot jbegin
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(4));
  if (!grouped) {
    HORA_TRY(launch_merge_topk(M, R, ws.ivf_cand.as<uint64_t>() + (int64_t)jbegin * R, ws.count.as<uint32_t>(),
                               width, 0, nullptr, nq, ws.ovf_flag.as<uint8_t>(),
                               ws.ovf_counter.as<uint32_t>(), s));
  } else {
    // merge probe slots in groups that fit one shared-memory sort
    int grp = std::max(1, (16384 - R) / R);
    for (int64_t j0 = jbegin; j0 < pmax; j0 += grp) {
      int gw = (int)(std::min<int64_t>(grp, pmax - j0) * R);
      HORA_TRY(ws.tmp_keys.reserve(sizeof(uint64_t) * nq * gw));
      HORA_CUDA_TRY(cudaMemcpy2DAsync(ws.tmp_keys.ptr, gw * 8, ws.ivf_cand.as<uint64_t>() + j0 * R, width * 8,
                                      gw * 8, nq, cudaMemcpyDeviceToDevice, s));
      HORA_TRY(launch_merge_topk(M, R, ws.tmp_keys.as<uint64_t>(), nullptr, gw, gw, nullptr, nq,
                                 ws.ovf_flag.as<uint8_t>(), ws.ovf_counter.as<uint32_t>(), s));
    }
  }
  return HORA_OK;
}

// k best of M (nq x R ADC keys): an exact FP32 rerank when R > k.
int ivf_finalize(hora_index *h, int64_t nq, int k, int R, const uint64_t *M, SearchWorkspace &ws,
                 uint64_t *d_best, cudaStream_t s) {
  if (R == k) {
    if (M != d_best)
      HORA_CUDA_TRY(cudaMemcpyAsync(d_best, M, sizeof(uint64_t) * nq * k, cudaMemcpyDeviceToDevice, s));
    return HORA_OK;
  }
  HORA_TRY(ws.tmp_keys.reserve(sizeof(uint64_t) * nq * R));
  if (h->metric == M_COS) HORA_TRY(ensure_norms(h, s));
  HORA_TRY(launch_rerank_exact(h->metric, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim,
                               ws.qnorm.as<float>(), h->xnorm.as<float>(), M, nq, R,
                               ws.tmp_keys.as<uint64_t>(), s));
  HORA_CUDA_TRY(cudaMemsetAsync(d_best, 0xff, sizeof(uint64_t) * nq * k, s));
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(4));
  HORA_TRY(launch_merge_topk(d_best, k, ws.tmp_keys.as<uint64_t>(), nullptr, R, R, nullptr, nq,
                             ws.ovf_flag.as<uint8_t>(), ws.ovf_counter.as<uint32_t>(), s));
  return HORA_OK;
}

int ivf_rerank_width(const hora_index *h, int k) { return h->ivf_rerank > k ? h->ivf_rerank : k; }

uint64_t *ivf_merge_buffer(SearchWorkspace &ws, int64_t nq, int R, uint64_t *d_best, int k) {
  if (R == k) return d_best;
  if (ws.best_r.reserve(sizeof(uint64_t) * nq * R) != HORA_OK) return nullptr;
  return ws.best_r.as<uint64_t>();
}

int ivf_search_keys(hora_index *h, int64_t nq, int k, int64_t nprobe, const uint32_t *d_nprobe,
                    SearchWorkspace &ws, uint64_t *d_best, cudaStream_t s) {
  if (!h->ivfs) return fail(HORA_ENOTBUILT, "index not built");
  const int pmax = ivf_pmax(h, nprobe);
  const int R = ivf_rerank_width(h, k);  // ADC candidates kept per query
  if (R > 1024) return fail(HORA_ECAP, "IVF-PQ: k (or rerank width) must be <= 1024");
  if (h->learned_nprobe && h->nprobe && !d_nprobe && nprobe == 0)
    return ivf_search_learned(h, nq, k, ws, d_best, s);
  HORA_TRY(ivf_probe(h, nq, pmax, ws, s));
  uint64_t *M = ivf_merge_buffer(ws, nq, R, d_best, k);
  if (!M) return fail(HORA_EOOM, "IVF-PQ: merge buffer");
  HORA_CUDA_TRY(cudaMemsetAsync(M, 0xff, sizeof(uint64_t) * nq * R, s));
  HORA_TRY(ivf_adc_merge(h, nq, pmax, 0, d_nprobe, R, M, ws, s));
  return ivf_finalize(h, nq, k, R, M, ws, d_best, s);
}

int ivf_layout(const hora_index *h, uint64_t *n_list, uint64_t *n_sub, uint64_t *sub_bits,
               uint64_t *dmax) {
  if (h->kind == HORA_INDEX_BRUTE_FORCE) return fail(HORA_EINVAL, "not a PQ index");
  int64_t sd = (int64_t)h->dim / (int64_t)h->ivf.n_sub;
  if (n_list) *n_list = h->ivf.n_kmeans_center;
  if (n_sub) *n_sub = h->ivf.n_sub;
  if (sub_bits) *sub_bits = h->ivf.sub_bits;
  if (dmax) *dmax = (uint64_t)(sd + (((int64_t)h->dim % sd) ? 1 : 0));
  return HORA_OK;
}

int ivf_export(const hora_index *h, float *centers, int64_t *offsets, int64_t *items,
               float *codebooks, uint8_t *codes, uint8_t *trained) {
  if (h->kind == HORA_INDEX_BRUTE_FORCE) return fail(HORA_EINVAL, "not a PQ index");
  if (!h->ivfs) return fail(HORA_ENOTBUILT, "index not built");
  const IvfState &v = *h->ivfs;
  const int64_t C = v.n_list, n = v.n_items;
  const int dexact = pq_dmax_of((int64_t)h->dim, v.n_sub);
  if (centers)
    HORA_CUDA_TRY(cudaMemcpy2D(centers, h->dim * 4, v.centers.ptr, h->ld * 4, h->dim * 4, C, cudaMemcpyDeviceToHost));
  if (offsets) std::copy(v.h_offsets.begin(), v.h_offsets.end(), offsets);
  if (items && n) {
    std::vector<uint32_t> t(n);
    HORA_CUDA_TRY(cudaMemcpy(t.data(), v.items.ptr, 4 * n, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) items[i] = t[i];
  }
  if (codebooks)
    HORA_CUDA_TRY(cudaMemcpy2D(codebooks, dexact * 4, v.books.ptr, v.dmax * 4, dexact * 4,
                               (size_t)C * v.n_sub * v.K, cudaMemcpyDeviceToHost));
  if (codes && n) HORA_CUDA_TRY(cudaMemcpy(codes, v.codes.ptr, n * v.n_sub, cudaMemcpyDeviceToHost));
  if (trained) std::copy(v.h_trained.begin(), v.h_trained.end(), trained);
  return HORA_OK;
}

// IVF-PQ block of the index file: layout sizes then the trained arrays.
int ivf_dump(const hora_index *h, FILE *f) {
  if (!h->ivfs) return HORA_OK;
  const IvfState &v = *h->ivfs;
  const int64_t C = v.n_list, n = v.n_items;
  const int dexact = pq_dmax_of((int64_t)h->dim, v.n_sub);
  std::vector<float> centers(C * h->dim), books(C * v.n_sub * v.K * dexact);
  std::vector<int64_t> offs(C + 1), items(n);
  std::vector<uint8_t> codes(n * v.n_sub), tr(C);
  HORA_TRY(ivf_export(h, centers.data(), offs.data(), items.data(), books.data(), codes.data(), tr.data()));
  int64_t hdr[3] = {C, n, v.n_sub};
  bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
            std::fwrite(centers.data(), 4, centers.size(), f) == centers.size() &&
            std::fwrite(books.data(), 4, books.size(), f) == books.size() &&
            std::fwrite(tr.data(), 1, tr.size(), f) == tr.size();
  return ok ? HORA_OK : fail(HORA_EIO, "write failed");
}

int ivf_load(hora_index *h, FILE *f) {
  int64_t hdr[3];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1) return fail(HORA_EIO, "corrupt index file");
  const int64_t C = hdr[0];
  if (C != (int64_t)h->ivf.n_kmeans_center || hdr[1] != h->n || hdr[2] != (int64_t)h->ivf.n_sub)
    return fail(HORA_EIO, "corrupt index file (IVF-PQ header)");
  const int dexact = pq_dmax_of((int64_t)h->dim, (int64_t)h->ivf.n_sub);
  const int64_t K = (int64_t)1 << h->ivf.sub_bits;
  std::vector<float> centers(C * h->dim), books(C * h->ivf.n_sub * K * dexact);
  std::vector<uint8_t> tr(C);
  bool ok = std::fread(centers.data(), 4, centers.size(), f) == centers.size() &&
            std::fread(books.data(), 4, books.size(), f) == books.size() &&
            std::fread(tr.data(), 1, tr.size(), f) == tr.size();
  if (!ok) return fail(HORA_EIO, "corrupt index file (IVF-PQ arrays)");
  HORA_TRY(ivf_set_codebooks(h, centers.data(), books.data()));
  // lists that were untrained stay untrained
  IvfState &v = *h->ivfs;
  for (int64_t c = 0; c < C; ++c) v.h_trained[c] = v.h_trained[c] && tr[c];
  HORA_CUDA_TRY(cudaMemcpy(v.trained.ptr, v.h_trained.data(), C, cudaMemcpyHostToDevice));
  return HORA_OK;
}

size_t ivf_device_bytes(const hora_index *h) {
  if (!h->ivfs) return 0;
  const IvfState &v = *h->ivfs;
  return v.centers.bytes + v.offsets.bytes + v.items.bytes + v.codes.bytes + v.books.bytes +
         v.trained.bytes + v.cnorm.bytes;
}

int ivf_info(const hora_index *h, std::string &out) {
  if (!h->ivfs) {
    out = "{\"trained\":false}";
    return HORA_OK;
  }
  const IvfState &v = *h->ivfs;
  int64_t empty = 0;
  for (int64_t c = 0; c < v.n_list; ++c) empty += v.h_offsets[c + 1] == v.h_offsets[c];
  out = "{\"n_list\":" + std::to_string(v.n_list) + ",\"n_sub\":" + std::to_string(v.n_sub) +
        ",\"sub_bits\":" + std::to_string(v.sub_bits) + ",\"max_list\":" + std::to_string(v.max_list) +
        ",\"empty_lists\":" + std::to_string(empty) + ",\"search_n_center\":" +
        std::to_string(h->ivf.search_n_center) + ",\"rerank\":" + std::to_string(h->ivf_rerank) +
        ",\"nprobe_model\":" + nprobe_model_info(h) + "}";
  return HORA_OK;
}

}  // namespace hora
