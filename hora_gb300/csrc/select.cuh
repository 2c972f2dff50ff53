// select.cuh — CTA-wide radix selection helpers.
#pragma once

#include "common.cuh"

namespace hora {

// Warp 0 scans a 256-bin histogram: finds the digit d whose cumulative count
// first reaches `rem` and writes d and the count of keys below d into
// out[0], out[1].  Lane l owns bins 8l..8l+7.
__device__ __forceinline__ void warp_find_digit(const uint32_t *hist, uint32_t rem, int *out) {
  const int lane = threadIdx.x & 31;
  uint32_t b[8], s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    b[i] = hist[lane * 8 + i];
    s += b[i];
  }
  uint32_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const uint32_t exc = inc - s;
  // the lane whose range contains the rem-th key
  const bool mine = exc < rem && inc >= rem;
  const unsigned who = __ballot_sync(0xffffffffu, mine);
  if (mine) {
    uint32_t run = exc;
    int d = lane * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (run + b[i] >= rem) {
        d = lane * 8 + i;
        break;
      }
      run += b[i];
    }
    out[0] = d;
    out[1] = (int)run;
  }
  if (who == 0 && lane == 31) {  // rem above the total (callers avoid it): last digit
    out[0] = 255;
    out[1] = (int)(inc - b[7]);
  }
}

constexpr int kSelBins = 2048;

// Warp 0: the bin whose cumulative count first reaches rem among nbins
// (32 times a power of two); out[0] = bin, out[1] = keys below it.  Lane l owns bins
// [l*nb, l*nb+nb) and sums them in a rotated order (conflict-free banks).
__device__ __forceinline__ void warp_find_bin(const uint32_t *hist, int nbins, uint32_t rem,
                                              int *out) {
  const int lane = threadIdx.x & 31, nb = nbins >> 5;  // nb: a power of two
  uint32_t s = 0;
#pragma unroll 8
  for (int i = 0; i < nb; ++i) s += hist[lane * nb + ((i + lane) & (nb - 1))];
  uint32_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const uint32_t exc = inc - s;
  const bool mine = exc < rem && inc >= rem;
  if (mine) {
    uint32_t run = exc;
    int d = lane * nb + nb - 1;
    for (int i = 0; i < nb; ++i) {
      const uint32_t b = hist[lane * nb + i];
      if (run + b >= rem) {
        d = lane * nb + i;
        break;
      }
      run += b;
    }
    out[0] = d;
    out[1] = (int)run;
  }
}

// Warp-wide minimum / maximum of a 64-bit value.
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y < v ? y : v;
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_max_u64_all(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  return v;
}

// Every lane of the warp: the digit of a 256-bin histogram whose cumulative
// count first reaches rem (1 <= rem <= the histogram's total) and the count
// of keys below it.  Lane l owns bins 8l..8l+7.
__device__ __forceinline__ void warp_digit_all(const uint32_t *hist, uint32_t rem, int &dig,
                                               uint32_t &below) {
  const int lane = threadIdx.x & 31;
  uint32_t b[8], s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    b[i] = hist[lane * 8 + i];
    s += b[i];
  }
  uint32_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const uint32_t exc = inc - s;
  const bool mine = exc < rem && inc >= rem;
  const unsigned who = __ballot_sync(0xffffffffu, mine);
  int d = lane * 8 + 7;
  uint32_t run = exc;
  if (mine) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (run + b[i] >= rem) {
        d = lane * 8 + i;
        break;
      }
      run += b[i];
    }
  }
  const int src = who ? __ffs(who) - 1 : 31;
  dig = __shfl_sync(0xffffffffu, d, src);
  below = __shfl_sync(0xffffffffu, run, src);
}

}  // namespace hora
