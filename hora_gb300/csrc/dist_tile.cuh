// dist_tile.cuh — exact FP32 distance tiles on the CUDA cores.
//
// One CTA of 256 threads scores a tile of 128 queries x 128 base rows; each
// thread owns an 8 x 8 register block (queries tq+16i, rows tn+16j).  The
// dimension is streamed in slabs of 32 floats through double-buffered
// cp.async staging.  Every (query, row) accumulator walks the dimensions in
// order 0..dim-1 with separately rounded __fsub_rn/__fmul_rn/__fadd_rn,
// which is exactly the reference's scalar loop (src/core/simd_metrics.rs:
// 30-33 dot, 60-66 L1, 96-102 squared L2): distances are bit-identical.
#pragma once

#include "common.cuh"

namespace hora {

constexpr int kTileQ = 128;
constexpr int kTileN = 128;
constexpr int kSlab = 32;
constexpr int kSkew = 4;                 // row pitch 36 floats: conflict-free LDS.128
constexpr int kPitch = kSlab + kSkew;
constexpr int kTileThreads = 256;
constexpr int kTileSmem = 2 * (kTileQ + kTileN) * kPitch * 4;  // 73,728 B

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Loads one 128-row x 32-column slab (columns [col0, col0+32)) of a row-major
// matrix with pitch ld floats (ld % 4 == 0; columns >= ld and rows >= nrows
// are zero-filled).
__device__ __forceinline__ void load_slab(float *dst, const float *src, int64_t ld, int64_t row0,
                                          int64_t nrows, int64_t col0, const int *rowmap) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int c = tid + r * kTileThreads;  // 0..1023
    int row = c >> 3, c4 = (c & 7) * 4;
    int64_t gr = row0 + row;
    int64_t gc = col0 + c4;
    bool ok = gr < nrows && gc < ld;
    int64_t srow = ok ? (rowmap ? rowmap[gr] : gr) : 0;
    const float *g = ok ? src + srow * ld + gc : src;
    cp_async16(dst + row * kPitch + c4, g, ok);
  }
}

template <int MT>
__device__ __forceinline__ float dist_op(float acc, float q, float x) {
  if (MT == M_L2) {
    float t = __fsub_rn(q, x);
    return __fadd_rn(acc, __fmul_rn(t, t));
  } else if (MT == M_L1) {
    return __fadd_rn(acc, fabsf(__fsub_rn(q, x)));
  } else {  // dot product (also the cosine numerator)
    return __fadd_rn(acc, __fmul_rn(q, x));
  }
}

// Scores the tile (queries [q0, q0+128) via qmap, rows [r0, r0+128)) into
// acc.  smem holds two stages of the query and row slabs.
template <int MT>
__device__ __forceinline__ void score_tile(float (&acc)[8][8], float *smem, const float *Q,
                                           int64_t ldq, int64_t nq_rows, int64_t q0,
                                           const int *qmap, const float *X, int64_t ldx,
                                           int64_t n_rows, int64_t r0, int64_t ld_common) {
  float *qs = smem;                        // [2][128][kPitch]
  float *xs = smem + 2 * kTileQ * kPitch;  // [2][128][kPitch]
  const int tid = threadIdx.x, tq = tid >> 4, tn = tid & 15;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

  const int nslab = (int)((ld_common + kSlab - 1) / kSlab);
  load_slab(qs, Q, ldq, q0, nq_rows, 0, qmap);
  load_slab(xs, X, ldx, r0, n_rows, 0, nullptr);
  cp_async_commit();
  for (int s = 0; s < nslab; ++s) {
    const int cur = s & 1;
    if (s + 1 < nslab) {
      load_slab(qs + (cur ^ 1) * kTileQ * kPitch, Q, ldq, q0, nq_rows, (int64_t)(s + 1) * kSlab, qmap);
      load_slab(xs + (cur ^ 1) * kTileN * kPitch, X, ldx, r0, n_rows, (int64_t)(s + 1) * kSlab, nullptr);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float *qc = qs + cur * kTileQ * kPitch;
    const float *xc = xs + cur * kTileN * kPitch;
#pragma unroll 2
    for (int kk = 0; kk < kSlab; kk += 4) {
      float4 qv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) qv[i] = *reinterpret_cast<const float4 *>(qc + (tq + 16 * i) * kPitch + kk);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float4 xv = *reinterpret_cast<const float4 *>(xc + (tn + 16 * j) * kPitch + kk);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          float a = acc[i][j];
          a = dist_op<MT>(a, qv[i].x, xv.x);
          a = dist_op<MT>(a, qv[i].y, xv.y);
          a = dist_op<MT>(a, qv[i].z, xv.z);
          a = dist_op<MT>(a, qv[i].w, xv.w);
          acc[i][j] = a;
        }
      }
    }
    __syncthreads();
  }
}

// Cosine from the dot product and the two f32 norms, as the oracle computes
// it: -(q.x) / (|q| * |x|), 0 when the denominator is 0.
__device__ __forceinline__ float cosine_from_dot(float dot, float qn, float xn) {
  float den = __fmul_rn(qn, xn);
  return den == 0.0f ? 0.0f : __fdiv_rn(-dot, den);
}

}  // namespace hora
