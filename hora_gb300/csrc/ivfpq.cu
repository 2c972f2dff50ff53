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
// block prefix, then an in-order warp scatter inside each block.
constexpr int kSortBlock = 1024;

__global__ void label_hist_kernel(const uint64_t *keys, const uint32_t *labels, int64_t n, int C,
                                  uint32_t *block_counts) {
  extern __shared__ uint32_t hist[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) hist[c] = 0;
  __syncthreads();
  int64_t lo = (int64_t)blockIdx.x * kSortBlock;
  for (int64_t i = lo + threadIdx.x; i < min(n, lo + kSortBlock); i += blockDim.x) {
    uint32_t l = keys ? key_row(keys[i]) : labels[i];
    atomicAdd(&hist[l], 1u);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) block_counts[(int64_t)blockIdx.x * C + c] = hist[c];
}

// per label: running offsets over blocks; totals -> counts[c]
__global__ void label_block_scan_kernel(uint32_t *block_counts, int64_t nblocks, int C,
                                        int64_t *counts) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  uint32_t run = 0;
  for (int64_t b = 0; b < nblocks; ++b) {
    uint32_t v = block_counts[b * C + c];
    block_counts[b * C + c] = run;
    run += v;
  }
  counts[c] = run;
}

// exclusive scan of C counts into offsets[0..C] (one CTA)
__global__ void offsets_scan_kernel(const int64_t *counts, int C, int64_t *offsets) {
  __shared__ int64_t part[1024];
  int t = threadIdx.x;
  int per = (C + blockDim.x - 1) / blockDim.x;
  int lo = t * per, hi = min(C, lo + per);
  int64_t s = 0;
  for (int c = lo; c < hi; ++c) s += counts[c];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int64_t run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      int64_t v = part[i];
      part[i] = run;
      run += v;
    }
    offsets[C] = run;
  }
  __syncthreads();
  int64_t run = part[t];
  for (int c = lo; c < hi; ++c) {
    offsets[c] = run;
    run += counts[c];
  }
}

__global__ void label_scatter_kernel(const uint64_t *keys, const uint32_t *labels, int64_t n, int C,
                                     const uint32_t *block_counts, const int64_t *offsets,
                                     uint32_t *members) {
  extern __shared__ uint32_t rank[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) rank[c] = 0;
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  int64_t lo = (int64_t)blockIdx.x * kSortBlock;
  int64_t hi = min(n, lo + kSortBlock);
  for (int64_t base = lo; base < hi; base += 32) {
    int64_t i = base + lane;
    bool ok = i < hi;
    uint32_t l = ok ? (keys ? key_row(keys[i]) : labels[i]) : 0xffffffffu;
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

// CTA-wide selection of the k smallest of L 32-bit order keys held in smem.
// The keys' range [kmin, kmax] comes first; the radix select then runs on
// key - kmin with its first 11-bit digit at the top of that range (plain
// shared atomics: the keys spread over the bins) and stops as soon as the
// k-th key's bin is taken whole; otherwise it resolves the k-th key exactly
// and ties at it go to the lowest positions.  sel receives the k positions
// (unordered).  L and k are uniform, 0 < k < L.  hist: kSelBins u32, zero on
// entry and on return; scratch: 48 ints.
__device__ void cta_select_k(const uint32_t *keys, int L, int k, int *sel, uint32_t *hist,
                             int *scratch) {
  // scratch: [0] remaining k, [1] digit, [2] below, [3] taken, [5] count at the digit,
  // [8..16) scan, [16..24) / [24..32) per-warp minima / maxima
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  uint32_t lo = 0xffffffffu, hi = 0;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const uint32_t v = keys[i];
    lo = min(lo, v);
    hi = max(hi, v);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if (lane == 0) {
    scratch[16 + warp] = (int)lo;
    scratch[24 + warp] = (int)hi;
  }
  if (threadIdx.x == 0) {
    scratch[0] = k;
    scratch[3] = 0;
  }
  __syncthreads();
  uint32_t kmin = 0xffffffffu, kmax = 0;
  for (int x = 0; x < nwarp; ++x) {
    kmin = min(kmin, (uint32_t)scratch[16 + x]);
    kmax = max(kmax, (uint32_t)scratch[24 + x]);
  }
  int shift = 32 - __clz((int)(kmax - kmin)) - 11;  // __clz(0) = 32
  shift = shift < 0 ? 0 : shift;
  uint32_t prefix = 0, mask = 0;
  bool whole = false;
  for (;;) {
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      const uint32_t d = keys[i] - kmin;
      if ((d & mask) == prefix) atomicAdd(&hist[(d >> shift) & (kSelBins - 1)], 1u);
    }
    __syncthreads();
    if (warp == 0) {
      warp_find_bin(hist, kSelBins, (uint32_t)scratch[0], scratch + 1);
      __syncwarp();
      const int d = scratch[1];
      const uint32_t at_d = hist[d];
      const int below = scratch[2];
      __syncwarp();
      for (int b = lane; b < kSelBins; b += 32) hist[b] = 0;
      if (lane == 0) {
        scratch[0] -= below;
        scratch[5] = (int)at_d;
      }
    }
    __syncthreads();
    prefix |= (uint32_t)scratch[1] << shift;
    mask |= (uint32_t)(kSelBins - 1) << shift;
    if (scratch[5] == scratch[0]) {  // every key in this bin is taken
      whole = true;
      break;
    }
    if (shift == 0) break;
    shift = shift >= 11 ? shift - 11 : 0;
  }
  if (whole) {
    // exactly k keys lie at or below the bin's largest d
    const uint32_t bound = prefix | ((1u << shift) - 1u);
    for (int i0 = 0; i0 < L; i0 += blockDim.x) {
      const int i = i0 + threadIdx.x;
      const bool p = i < L && keys[i] - kmin <= bound;
      const unsigned pm = __ballot_sync(0xffffffffu, p);
      if (pm) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&scratch[3], __popc(pm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (p) sel[base + __popc(pm & ((1u << lane) - 1u))] = i;
      }
    }
    __syncthreads();
    return;
  }
  prefix += kmin;  // the k-th key itself
  const uint32_t kth = prefix;
  const int need_eq = scratch[0];  // keys equal to kth that are taken (>= 1)
  const bool all_eq = scratch[5] == need_eq;
  // keys below kth (and, when every key equal to kth is taken, those too)
  for (int i0 = 0; i0 < L; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    const uint32_t v = i < L ? keys[i] : 0xffffffffu;
    const bool p = i < L && (v < kth || (all_eq && v == kth));
    const unsigned pm = __ballot_sync(0xffffffffu, p);
    if (pm) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&scratch[3], __popc(pm));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (p) sel[base + __popc(pm & ((1u << lane) - 1u))] = i;
    }
  }
  if (all_eq) {
    __syncthreads();
    return;
  }
  __syncthreads();
  const int base_lt = scratch[3];
  // keys equal to kth in position order: chunked block scan
  int run = 0;
  const int nw = blockDim.x >> 5;
  for (int i0 = 0; i0 < L && run < need_eq; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    const bool f = i < L && keys[i] == kth;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if (lane == 0) scratch[8 + warp] = __popc(b);
    __syncthreads();
    int before = run;
    for (int x = 0; x < warp; ++x) before += scratch[8 + x];
    int total = 0;
    for (int x = 0; x < nw; ++x) total += scratch[8 + x];
    if (f) {
      const int r = before + __popc(b & ((1u << lane) - 1u));
      if (r < need_eq) sel[base_lt + r] = i;
    }
    run += total;
    __syncthreads();
  }
}

constexpr int kAdcThreads = 256;
constexpr int kAdcChunk = 2048;

// The sum over subspaces of LUT[m][code[m]] in subspace order (pq_idx.rs
// 180-186), with the code row read VB bytes at a time (VB divides M and the
// row pitch, so every load is aligned); KC = K when it is a compile-time 256.
template <int VB, int KC>
__device__ __forceinline__ float adc_row(const uint8_t *code, const float *lut, int M, int Kr) {
  const int K = KC ? KC : Kr;  // a constant K folds the table offsets into the loads
  float d = 0.0f;
  if (VB == 16) {
    const uint4 *p = reinterpret_cast<const uint4 *>(code);
    for (int g = 0; g < M / 16; ++g) {
      const uint4 w = __ldg(p + g);
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const uint32_t wt = t < 4 ? w.x : t < 8 ? w.y : t < 12 ? w.z : w.w;
        d = __fadd_rn(d, lut[(g * 16 + t) * K + ((wt >> (8 * (t & 3))) & 255u)]);
      }
    }
  } else if (VB == 8) {
    const uint2 *p = reinterpret_cast<const uint2 *>(code);
    for (int g = 0; g < M / 8; ++g) {
      const uint2 w = __ldg(p + g);
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const uint32_t wt = t < 4 ? w.x : w.y;
        d = __fadd_rn(d, lut[(g * 8 + t) * K + ((wt >> (8 * (t & 3))) & 255u)]);
      }
    }
  } else if (VB == 4) {
    const uint32_t *p = reinterpret_cast<const uint32_t *>(code);
    for (int g = 0; g < M / 4; ++g) {
      const uint32_t w = __ldg(p + g);
#pragma unroll
      for (int t = 0; t < 4; ++t) d = __fadd_rn(d, lut[(g * 4 + t) * K + ((w >> (8 * t)) & 255u)]);
    }
  } else {
    for (int m = 0; m < M; ++m) d = __fadd_rn(d, lut[m * K + __ldg(code + m)]);
  }
  return d;
}

// LUT[m][j] = metric(z[range_m], C[m][j]) in t order (pq_idx.rs:170-179):
// Euclidean inside IVF-PQ, the build metric for a flat PQIndex; the DM floats
// of a codeword are one aligned vector load.
template <int MT, int DM>
__device__ __forceinline__ float lut_entry(const float *cj, const float *zq, int len) {
  float c[DM];
  if (DM % 4 == 0) {
#pragma unroll
    for (int u = 0; u < DM; u += 4) {
      const float4 t = __ldg(reinterpret_cast<const float4 *>(cj + u));
      c[u] = t.x;
      c[u + 1] = t.y;
      c[u + 2] = t.z;
      c[u + 3] = t.w;
    }
  } else if (DM == 2) {
    const float2 t = __ldg(reinterpret_cast<const float2 *>(cj));
    c[0] = t.x;
    c[DM - 1] = t.y;
  } else {
#pragma unroll
    for (int u = 0; u < DM; ++u) c[u] = __ldg(cj + u);
  }
  float s = 0.0f;
#pragma unroll
  for (int u = 0; u < DM; ++u)
    if (u < len) s = dist_op<MT>(s, zq[u], c[u]);
  return s;
}

// One CTA handles `per` consecutive (query, list) pairs (sorted by list):
// LUT, ADC scan of the list in chunks, and the pair's kk best (distance,
// row) keys -> cand[(q * pmax + slot) * kk ...].
template <int DM, int VB>
__global__ void __launch_bounds__(kAdcThreads) adc_scan_kernel(
    const float *Q, int64_t ldq, const float *centers, int64_t ldc, const float *books,
    const uint8_t *codes, const uint32_t *items, const int64_t *offs, const uint8_t *trained,
    const uint32_t *pq, const uint32_t *pc, const uint32_t *pslot, int64_t npairs, int per, int M,
    int K, const int *sb, const int *sl, int mt, int kk, int pmax, uint64_t *cand) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float *lut = reinterpret_cast<float *>(smraw);                       // M x K
  uint32_t *hist = reinterpret_cast<uint32_t *>(lut + M * K);          // kSelBins
  uint32_t *dkeys = hist + kSelBins;                                   // kAdcChunk + kk
  uint32_t *rows = dkeys + kAdcChunk + kk;                             // kAdcChunk + kk
  int *sel = reinterpret_cast<int *>(rows + kAdcChunk + kk);           // kk
  int *scratch = sel + kk;                                             // 48
  int *sbs = scratch + 48;                                             // M subspace starts
  int *sls = sbs + M;                                                  // M subspace lengths
  __shared__ __align__(16) float zq[1024];
  for (int b = threadIdx.x; b < kSelBins; b += blockDim.x) hist[b] = 0;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    sbs[m] = sb[m];
    sls[m] = sl[m];
  }
  const int kbits = 31 - __clz(K);  // K = 2^sub_bits
  for (int64_t pi = (int64_t)blockIdx.x * per; pi < min(npairs, (int64_t)(blockIdx.x + 1) * per); ++pi) {
    const int64_t q = pq[pi];
    const int c = (int)pc[pi];
    const int slot = (int)pslot[pi];
    uint64_t *out = cand + (q * pmax + slot) * kk;
    const int64_t lo = offs[c], L = offs[c + 1] - lo;
    if (!trained[c] || L == 0) {
      for (int r = threadIdx.x; r < kk; r += blockDim.x) out[r] = kEmptyKey;
      continue;
    }
    // z = q - c_list over the covered dimensions (pq_idx.rs:158-161)
    const int dcov = sb[M - 1] + sl[M - 1];
    __syncthreads();  // the previous pair is done with zq and the LUT
    for (int t = threadIdx.x; t < dcov; t += blockDim.x)
      zq[t] = __fsub_rn(Q[q * ldq + t], centers[(int64_t)c * ldc + t]);
    __syncthreads();
    const float *book = books + (int64_t)c * M * K * DM;
    if (DM == 4 && mt == M_L2) {
      // 8 codewords' loads in flight per thread before any entry is computed
      const float4 *b4 = reinterpret_cast<const float4 *>(book);
      const int MK = M * K;
      for (int e0 = threadIdx.x; e0 < MK; e0 += 8 * kAdcThreads) {
        float4 cv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * kAdcThreads;
          if (e < MK) cv[u] = __ldg(b4 + e);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * kAdcThreads;
          if (e < MK) {
            const int m = e >> kbits, len = sls[m];
            const float *z = zq + sbs[m];
            const float cw[4] = {cv[u].x, cv[u].y, cv[u].z, cv[u].w};
            float acc = 0.0f;
#pragma unroll
            for (int t = 0; t < 4; ++t)
              if (t < len) acc = dist_op<M_L2>(acc, z[t], cw[t]);
            lut[e] = acc;
          }
        }
      }
    } else if (mt == M_L2) {
      for (int e = threadIdx.x; e < M * K; e += blockDim.x) {
        const int m = e >> kbits;
        lut[e] = lut_entry<M_L2, DM>(book + (int64_t)e * DM, zq + sbs[m], sls[m]);
      }
    } else if (mt == M_L1) {
      for (int e = threadIdx.x; e < M * K; e += blockDim.x) {
        const int m = e >> kbits;
        lut[e] = lut_entry<M_L1, DM>(book + (int64_t)e * DM, zq + sbs[m], sls[m]);
      }
    } else {
      for (int e = threadIdx.x; e < M * K; e += blockDim.x) {
        const int m = e >> kbits;
        lut[e] = lut_entry<M_IP, DM>(book + (int64_t)e * DM, zq + sbs[m], sls[m]);
      }
    }
    __syncthreads();
    // scan in chunks; running kk best kept at the head of dkeys/rows
    int held = 0;
    const uint8_t *lcodes = codes + lo * M;
    for (int64_t c0 = 0; c0 < L; c0 += kAdcChunk) {
      const int ch = (int)(kAdcChunk < L - c0 ? (int64_t)kAdcChunk : L - c0);
      for (int i = threadIdx.x; i < ch; i += blockDim.x) {
        const float d = K == 256 ? adc_row<VB, 256>(lcodes + (c0 + i) * M, lut, M, K)
                                 : adc_row<VB, 0>(lcodes + (c0 + i) * M, lut, M, K);
        dkeys[held + i] = f2ord(d);
        rows[held + i] = items[lo + c0 + i];
      }
      __syncthreads();
      const int tot = held + ch;
      if (tot <= kk) {
        held = tot;
        continue;
      }
      cta_select_k(dkeys, tot, kk, sel, hist, scratch);
      // gather the selection to the head (through registers: sel is unordered)
      static_assert(kAdcThreads * 4 >= 1024, "kk <= 1024 is held in 4 registers a thread");
      uint32_t kv[4], rv[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int r = threadIdx.x + t * kAdcThreads;
        if (r < kk) {
          kv[t] = dkeys[sel[r]];
          rv[t] = rows[sel[r]];
        }
      }
      __syncthreads();
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int r = threadIdx.x + t * kAdcThreads;
        if (r < kk) {
          dkeys[r] = kv[t];
          rows[r] = rv[t];
        }
      }
      held = kk;
      __syncthreads();
    }
    for (int r = threadIdx.x; r < kk; r += blockDim.x)
      out[r] = r < held ? (((uint64_t)dkeys[r] << 32) | rows[r]) : kEmptyKey;
  }
}

// ---------------------------------------------------------------------------
// host side

int sort_labels(const uint64_t *keys, const uint32_t *labels, int64_t n, int C,
                       DevBuf &blk, DevBuf &counts, int64_t *d_offsets, uint32_t *d_members,
                       cudaStream_t s) {
  int64_t nb = ceil_div(n, kSortBlock);
  HORA_TRY(blk.reserve(sizeof(uint32_t) * nb * C));
  HORA_TRY(counts.reserve(sizeof(int64_t) * C));
  int smem = C * 4;
  HORA_SMEM_ATTR(label_hist_kernel, smem);
  HORA_SMEM_ATTR(label_scatter_kernel, smem);
  {
    ProfScope ps("ivf_sort", s);
    label_hist_kernel<<<(unsigned)nb, 256, smem, s>>>(keys, labels, n, C, blk.as<uint32_t>());
    HORA_LAUNCHED();
    label_block_scan_kernel<<<ceil_div(C, 256), 256, 0, s>>>(blk.as<uint32_t>(), nb, C, counts.as<int64_t>());
    HORA_LAUNCHED();
    offsets_scan_kernel<<<1, 1024, 0, s>>>(counts.as<int64_t>(), C, d_offsets);
    HORA_LAUNCHED();
    label_scatter_kernel<<<(unsigned)nb, 256, smem, s>>>(keys, labels, n, C, blk.as<uint32_t>(),
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
  h->built = true;
  return HORA_OK;
}

template <int DM, int VB>
static int launch_adc_vb(IvfState &v, SearchWorkspace &ws, const float *Q, int64_t ldq, int64_t ldc,
                         int64_t npairs, int per, int kk, int pmax, uint64_t *cand, cudaStream_t s) {
  // LUT, histogram, keys + rows of a chunk and the carried kk, selection, scratch
  size_t smem = sizeof(float) * v.n_sub * v.K + sizeof(uint32_t) * kSelBins +
                2 * sizeof(uint32_t) * (kAdcChunk + kk) + sizeof(int) * kk + sizeof(int) * 48 +
                2 * sizeof(int) * v.n_sub;
  if (smem > 200 * 1024) return fail(HORA_ECAP, "IVF-PQ: LUT too large for shared memory");
  HORA_SMEM_ATTR((adc_scan_kernel<DM, VB>), smem);
  unsigned grid = (unsigned)ceil_div(npairs, per);
  if (grid == 0) return HORA_OK;
  ProfScope ps("adc_scan", s);
  adc_scan_kernel<DM, VB><<<grid, kAdcThreads, smem, s>>>(
      Q, ldq, v.centers.as<float>(), ldc, v.books.as<float>(), v.codes.as<uint8_t>(),
      v.items.as<uint32_t>(), v.offsets.as<int64_t>(), v.trained.as<uint8_t>(), ws.pair_q.as<uint32_t>(),
      ws.pair_c.as<uint32_t>(), ws.pair_slot.as<uint32_t>(), npairs, per, (int)v.n_sub, (int)v.K,
      v.sub_begin_d.as<int>(), v.sub_len_d.as<int>(), v.pq_metric, kk, pmax, cand);
  HORA_LAUNCHED();
  return HORA_OK;
}

// Code rows are n_sub bytes apart: the widest load that divides n_sub.
template <int DM>
static int launch_adc(IvfState &v, SearchWorkspace &ws, const float *Q, int64_t ldq, int64_t ldc,
                      int64_t npairs, int per, int kk, int pmax, uint64_t *cand, cudaStream_t s) {
  if (v.n_sub % 16 == 0) return launch_adc_vb<DM, 16>(v, ws, Q, ldq, ldc, npairs, per, kk, pmax, cand, s);
  if (v.n_sub % 8 == 0) return launch_adc_vb<DM, 8>(v, ws, Q, ldq, ldc, npairs, per, kk, pmax, cand, s);
  if (v.n_sub % 4 == 0) return launch_adc_vb<DM, 4>(v, ws, Q, ldq, ldc, npairs, per, kk, pmax, cand, s);
  return launch_adc_vb<DM, 1>(v, ws, Q, ldq, ldc, npairs, per, kk, pmax, cand, s);
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
  HORA_TRY(ws.pair_cnt.reserve(sizeof(int64_t) * (C + 1) * 2));
  HORA_TRY(ws.pair_off.reserve(sizeof(int64_t) * (C + 1)));
  int64_t *cnt = ws.pair_cnt.as<int64_t>();
  int64_t *cursor = cnt + (C + 1);
  HORA_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (C + 1) * 2, s));
  const int64_t tot = nq * pmax;
  {
    ProfScope ps("ivf_pairs", s);
    pair_hist_kernel<<<ceil_div(tot, 256), 256, 0, s>>>(ws.probes.as<uint64_t>(), nq, pmax, jbegin,
                                                       d_nprobe, C, cnt);
    HORA_LAUNCHED();
    offsets_scan_kernel<<<1, 1024, 0, s>>>(cnt, C, ws.pair_off.as<int64_t>());
    HORA_LAUNCHED();
  }
  int64_t npairs = nq * (pmax - jbegin);
  if (d_nprobe) {
    HORA_CUDA_TRY(cudaMemcpyAsync(&npairs, ws.pair_off.as<int64_t>() + C, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (npairs <= 0) return HORA_OK;
  HORA_TRY(ws.pair_q.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  HORA_TRY(ws.pair_c.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  HORA_TRY(ws.pair_slot.reserve(sizeof(uint32_t) * std::max<int64_t>(tot, 1)));
  {
    ProfScope ps("ivf_pairs", s);
    pair_scatter_kernel<<<ceil_div(tot, 256), 256, 0, s>>>(
        ws.probes.as<uint64_t>(), nq, pmax, jbegin, d_nprobe, C, ws.pair_off.as<int64_t>(), cursor,
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
  const int per = 4;
  switch (v.dmax) {
    case 1: HORA_TRY(launch_adc<1>(v, ws, Q, h->ld, h->ld, npairs, per, R, pmax, ws.ivf_cand.as<uint64_t>(), s)); break;
    case 2: HORA_TRY(launch_adc<2>(v, ws, Q, h->ld, h->ld, npairs, per, R, pmax, ws.ivf_cand.as<uint64_t>(), s)); break;
    case 4: HORA_TRY(launch_adc<4>(v, ws, Q, h->ld, h->ld, npairs, per, R, pmax, ws.ivf_cand.as<uint64_t>(), s)); break;
    case 8: HORA_TRY(launch_adc<8>(v, ws, Q, h->ld, h->ld, npairs, per, R, pmax, ws.ivf_cand.as<uint64_t>(), s)); break;
    default: HORA_TRY(launch_adc<16>(v, ws, Q, h->ld, h->ld, npairs, per, R, pmax, ws.ivf_cand.as<uint64_t>(), s)); break;
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
