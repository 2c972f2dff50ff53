// bf_fp32.cu — exact FP32 scoring kernels on the CUDA cores.
//
// dist_tile_kernel is the workhorse of every exact path:
//   TILE_FILTER  brute-force scan (BruteForceIndex::node_search_k,
//                src/index/bruteforce_idx.rs:47-73): a row becomes a
//                candidate of query q when its (distance, row) key beats the
//                k-th best key found so far for q;
//   TILE_DENSE   the first chunk of a scan: every row is a candidate;
//   TILE_ARGMIN  k-means assignment (Kmeans::search_data, src/core/kmeans.rs:
//                127-148): strict '<' from centre 0 == smallest (d, row) key;
//   TILE_DIST    dense distances (coarse-centre probing, pq_idx.rs:416-421).
#include <algorithm>

#include "dist_tile.cuh"
#include "internal.h"

namespace hora {

template <int MT, int MODE>
__global__ void __launch_bounds__(kTileThreads, 1) dist_tile_kernel(TileParams p) {
  extern __shared__ __align__(16) float smem[];
  const int tid = threadIdx.x, tq = tid >> 4, tn = tid & 15;
  const int64_t q0 = (int64_t)blockIdx.x * kTileQ;
  float acc[8][8];

  // query ids and per-query state of this thread's 8 queries
  int64_t qid[8];
  float qn[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t q = q0 + tq + 16 * i;
    qid[i] = q < p.nq ? (p.qmap ? p.qmap[q] : q) : -1;
    qn[i] = (MT == M_COS && qid[i] >= 0) ? p.qnorm[qid[i]] : 0.0f;
  }

  if (MODE == TILE_ARGMIN) {
    uint64_t best[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) best[i] = kEmptyKey;
    for (int64_t r0 = p.r_begin; r0 < p.r_end; r0 += kTileN) {
      score_tile<MT>(acc, smem, p.Q, p.ldq, p.nq, q0, p.qmap, p.X, p.ldx, p.r_end, r0, p.ld);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        int64_t row = r0 + tn + 16 * j;
        if (row >= p.r_end) continue;
        float xn = MT == M_COS ? p.xnorm[row] : 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          float d = MT == M_COS ? cosine_from_dot(acc[i][j], qn[i], xn) : acc[i][j];
          uint64_t key = make_key(d, (uint32_t)row);
          best[i] = key < best[i] ? key : best[i];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
#pragma unroll
      for (int off = 8; off >= 1; off >>= 1) {
        uint64_t o = __shfl_xor_sync(0xffffffffu, best[i], off);
        best[i] = o < best[i] ? o : best[i];
      }
      if (tn == 0 && qid[i] >= 0) p.out_key[qid[i]] = best[i];
    }
    return;
  }

  const int64_t r0 = p.r_begin + (int64_t)blockIdx.y * kTileN;
  score_tile<MT>(acc, smem, p.Q, p.ldq, p.nq, q0, p.qmap, p.X, p.ldx, p.r_end, r0, p.ld);

  uint64_t tau[8];
  if (MODE == TILE_FILTER) {
#pragma unroll
    for (int i = 0; i < 8; ++i) tau[i] = qid[i] >= 0 ? p.best[qid[i] * p.k + (p.k - 1)] : 0ull;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    int64_t row = r0 + tn + 16 * j;
    if (row >= p.r_end) continue;
    float xn = MT == M_COS ? p.xnorm[row] : 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (qid[i] < 0) continue;
      float d = MT == M_COS ? cosine_from_dot(acc[i][j], qn[i], xn) : acc[i][j];
      if (MODE == TILE_DIST) {
        p.out_dist[qid[i] * p.ldo + (row - p.r_begin)] = d;
      } else {
        uint64_t key = make_key(d, (uint32_t)row);
        if (MODE == TILE_DENSE) {
          p.cand[qid[i] * p.cap + (row - p.r_begin)] = key;
        } else if (key < tau[i]) {
          uint32_t slot = atomicAdd(p.count + qid[i], 1u);
          if (slot < (uint32_t)p.cap) p.cand[qid[i] * p.cap + slot] = key;
        }
      }
    }
  }
}

template <int MT, int MODE>
static int launch_one(const TileParams &p, cudaStream_t s) {
  HORA_SMEM_ATTR((dist_tile_kernel<MT, MODE>), kTileSmem);
  dim3 grid(ceil_div(p.nq, kTileQ), 1);
  if (MODE != TILE_ARGMIN) grid.y = ceil_div(p.r_end - p.r_begin, kTileN);
  if (grid.x == 0 || grid.y == 0) return HORA_OK;
  if (grid.y > 65535) return fail(HORA_ECAP, "dist_tile: chunk too large for one launch");
  ProfScope ps(MODE == TILE_ARGMIN ? "fp32_tile_argmin"
               : MODE == TILE_DIST ? "fp32_tile_dist" : "fp32_tile_scan", s);
  dist_tile_kernel<MT, MODE><<<grid, kTileThreads, kTileSmem, s>>>(p);
  HORA_LAUNCHED();
  return HORA_OK;
}

template <int MT>
static int launch_mode(int mode, const TileParams &p, cudaStream_t s) {
  switch (mode) {
    case TILE_FILTER: return launch_one<MT, TILE_FILTER>(p, s);
    case TILE_DENSE: return launch_one<MT, TILE_DENSE>(p, s);
    case TILE_ARGMIN: return launch_one<MT, TILE_ARGMIN>(p, s);
    case TILE_DIST: return launch_one<MT, TILE_DIST>(p, s);
  }
  return fail(HORA_EINVAL, "dist_tile: bad mode");
}

int launch_dist_tile(int metric, int mode, const TileParams &p, cudaStream_t s) {
  if (p.ld % 4 || p.ldq % 4 || p.ldx % 4) return fail(HORA_EINVAL, "dist_tile: pitch not a multiple of 4");
  switch (metric) {
    case M_L2: return launch_mode<M_L2>(mode, p, s);
    case M_L1: return launch_mode<M_L1>(mode, p, s);
    case M_IP: return launch_mode<M_IP>(mode, p, s);
    case M_COS: return launch_mode<M_COS>(mode, p, s);
  }
  return fail(HORA_EMETRIC, "unknown method");
}

// ---- row norms: f32 sqrt(sum x^2) in reference order, and f64 sum x^2 ----------
__global__ void row_norms_kernel(const float *X, int64_t n, int64_t ld, int64_t dim, float *nf,
                                 double *sq) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float *x = X + r * ld;
  float s = 0.0f;
  double s64 = 0.0;
  for (int64_t t = 0; t < dim; ++t) {
    float v = x[t];
    s = __fadd_rn(s, __fmul_rn(v, v));
    s64 += (double)v * (double)v;
  }
  if (nf) nf[r] = __fsqrt_rn(s);
  if (sq) sq[r] = s64;
}

int launch_row_norms(const float *X, int64_t n, int64_t ld, int64_t dim, float *nf, double *sq,
                     cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  row_norms_kernel<<<ceil_div(n, 256), 256, 0, s>>>(X, n, ld, dim, nf, sq);
  HORA_LAUNCHED();
  return HORA_OK;
}

// Query staging in one pass: each thread copies its row from src (pitch
// lds) to dst (pitch ld, zero padding; src may alias dst), flags a NaN / Inf
// element and computes the norms in the same order as row_norms_kernel.
__global__ void stage_rows_kernel(const float *src, int64_t lds, int64_t n, int64_t dim, int64_t ld,
                                  float *dst, uint32_t *flag, float *nf, double *sq) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float *x = src + r * lds;
  float *y = dst + r * ld;
  float s = 0.0f;
  double s64 = 0.0;
  bool bad = false;
  int64_t t = 0;
  if ((lds & 3) == 0 && ((uintptr_t)src & 15) == 0) {
    // 16-byte loads, eight in flight: the sums still run over the
    // dimensions in order
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    float4 *y4 = reinterpret_cast<float4 *>(y);
    for (; t + 32 <= dim; t += 32) {
      float4 w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) w[u] = x4[t / 4 + u];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        y4[t / 4 + u] = w[u];
        const float e[4] = {w[u].x, w[u].y, w[u].z, w[u].w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          bad |= !isfinite(e[i]);
          s = __fadd_rn(s, __fmul_rn(e[i], e[i]));
          s64 += (double)e[i] * (double)e[i];
        }
      }
    }
  }
  for (; t < dim; ++t) {
    const float v = x[t];
    y[t] = v;
    bad |= !isfinite(v);
    s = __fadd_rn(s, __fmul_rn(v, v));
    s64 += (double)v * (double)v;
  }
  for (t = dim; t < ld; ++t) y[t] = 0.0f;
  if (bad && flag) atomicOr(flag, 1u);
  if (nf) nf[r] = __fsqrt_rn(s);
  if (sq) sq[r] = s64;
}

int launch_stage_rows(const float *src, int64_t lds, int64_t n, int64_t dim, int64_t ld, float *dst,
                      uint32_t *flag, float *nf, double *sq, cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  stage_rows_kernel<<<ceil_div(n, 32), 32, 0, s>>>(src, lds, n, dim, ld, dst, flag, nf, sq);
  HORA_LAUNCHED();
  return HORA_OK;
}

__global__ void check_finite_kernel(const float *X, int64_t n, int64_t ld, int64_t dim,
                                    uint32_t *flag) {
  int64_t total = n * dim;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v = X[(i / dim) * ld + (i % dim)];
    if (!isfinite(v)) {
      atomicOr(flag, 1u);
      return;
    }
  }
}

int launch_check_finite(const float *X, int64_t n, int64_t ld, int64_t dim, uint32_t *flag,
                        cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  int64_t total = n * dim;
  int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 152 * 16);
  check_finite_kernel<<<blocks, 256, 0, s>>>(X, n, ld, dim, flag);
  HORA_LAUNCHED();
  return HORA_OK;
}

// Exact FP32 distance of each query's R candidate rows (reference op order:
// one running sum over the dimensions in order, bit-identical to the scan
// kernel and the reference's scalar loops).  One CTA per query with
// ceil(R / 32) warps (at most kRrMaxWarps), so that R = 132 takes one round of
// five warps rather than two rounds of four; a warp takes 32 candidates at a
// time and reads their rows 64 dimensions at a time (two rows per coalesced
// 512-byte load) into a padded shared tile (row stride 65 floats:
// conflict-free column reads); each lane then sums its own row from the tile
// in dimension order.
constexpr int kRrMaxWarps = 8, kRrSlab = 64;
// With count, query q's list holds min(count[q], R) keys (the rest of its R
// slots are neither read nor written); in and outk may be the same buffer.
// With order, CTA b takes query order[b] (a permutation of the queries):
// queries whose candidates share rows run side by side and meet them in L2.
template <int MT>
__global__ void __launch_bounds__(kRrMaxWarps * 32) rerank_exact_kernel(
    const float *Q, int64_t ld, const float *X, int64_t dim, const float *qnorm, const float *xnorm,
    const uint64_t *in, int R, const uint32_t *count, const uint32_t *order, uint64_t *outk) {
  extern __shared__ float rr_smem[];  // per warp a 32 x (kRrSlab + 1) tile, then the query row
  const int nw = blockDim.x >> 5;
  float *qs = rr_smem + nw * 32 * (kRrSlab + 1);
  const int64_t q = order ? (int64_t)order[blockIdx.x] : (int64_t)blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t t = threadIdx.x; t < ld; t += blockDim.x) qs[t] = Q[q * ld + t];
  __syncthreads();
  const int64_t n4 = (dim + 3) / 4;  // the zero-padded columns up to 4*n4 add exact zeros
  float(*tw)[kRrSlab + 1] = reinterpret_cast<float(*)[kRrSlab + 1]>(rr_smem + warp * 32 * (kRrSlab + 1));
  const int half = lane >> 4, c4 = lane & 15;
  const int Rq = count ? (int)min(count[q], (uint32_t)R) : R;
  for (int r0 = warp * 32; r0 < Rq; r0 += nw * 32) {
    const int r = r0 + lane;
    const uint64_t key = r < Rq ? in[q * R + r] : kEmptyKey;
    float s = 0.0f;
    for (int64_t d0 = 0; d0 < 4 * n4; d0 += kRrSlab) {
      const int w = (int)(4 * n4 - d0 < kRrSlab ? 4 * n4 - d0 : kRrSlab);  // multiple of 4
      // 8 rows' loads in flight per lane before any is stored
      for (int jb = 0; jb < 16; jb += 8) {
        float4 vv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int jj = 2 * (jb + u) + half;
          const uint64_t kj = __shfl_sync(0xffffffffu, key, jj);
          vv[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (kj != kEmptyKey && 4 * c4 < w)
            vv[u] = __ldg(reinterpret_cast<const float4 *>(X + (int64_t)key_row(kj) * ld + d0) + c4);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int jj = 2 * (jb + u) + half;
          if (4 * c4 < w) {
            tw[jj][4 * c4] = vv[u].x;
            tw[jj][4 * c4 + 1] = vv[u].y;
            tw[jj][4 * c4 + 2] = vv[u].z;
            tw[jj][4 * c4 + 3] = vv[u].w;
          }
        }
      }
      __syncwarp();
      constexpr int OP = MT == M_COS ? M_IP : MT;
      for (int t = 0; t < w; ++t) s = dist_op<OP>(s, qs[d0 + t], tw[lane][t]);
      __syncwarp();
    }
    if (r < Rq) {
      if (key == kEmptyKey) {
        outk[q * R + r] = kEmptyKey;
      } else {
        const uint32_t row = key_row(key);
        if (MT == M_COS) s = cosine_from_dot(s, qnorm[q], xnorm[row]);
        outk[q * R + r] = make_key(s, row);
      }
    }
  }
}

int launch_rerank_exact(int metric, const float *Q, int64_t ld, const float *X, int64_t dim,
                        const float *qnorm, const float *xnorm, const uint64_t *in, int64_t nq,
                        int R, uint64_t *out, cudaStream_t s, const uint32_t *count, const uint32_t *order) {
  if (nq <= 0) return HORA_OK;
  if (ld % 4) return fail(HORA_EINVAL, "rerank: pitch not a multiple of 4");
  ProfScope ps("rerank_exact", s);
  unsigned g = (unsigned)nq;
  const int nw = count ? kRrMaxWarps : std::max(1, std::min(kRrMaxWarps, (R + 31) / 32));
  const int T = nw * 32;
  // the warps' tiles and the query row in dynamic shared memory
  const size_t qb = sizeof(float) * ((size_t)nw * 32 * (kRrSlab + 1) + (size_t)ld);
  if (qb > 200 * 1024) return fail(HORA_EINVAL, "rerank: dimension too large");
  HORA_SMEM_ATTR(rerank_exact_kernel<M_L2>, qb);
  HORA_SMEM_ATTR(rerank_exact_kernel<M_L1>, qb);
  HORA_SMEM_ATTR(rerank_exact_kernel<M_IP>, qb);
  HORA_SMEM_ATTR(rerank_exact_kernel<M_COS>, qb);
  switch (metric) {
    case M_L2: rerank_exact_kernel<M_L2><<<g, T, qb, s>>>(Q, ld, X, dim, qnorm, xnorm, in, R, count, order, out); break;
    case M_L1: rerank_exact_kernel<M_L1><<<g, T, qb, s>>>(Q, ld, X, dim, qnorm, xnorm, in, R, count, order, out); break;
    case M_IP: rerank_exact_kernel<M_IP><<<g, T, qb, s>>>(Q, ld, X, dim, qnorm, xnorm, in, R, count, order, out); break;
    case M_COS: rerank_exact_kernel<M_COS><<<g, T, qb, s>>>(Q, ld, X, dim, qnorm, xnorm, in, R, count, order, out); break;
    default: return fail(HORA_EMETRIC, "unknown method");
  }
  HORA_LAUNCHED();
  return HORA_OK;
}

}  // namespace hora
