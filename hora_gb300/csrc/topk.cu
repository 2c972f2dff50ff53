// topk.cu — k-best selection.
//
// The reference keeps a bounded std BinaryHeap per query (push, pop when
// longer than k: src/index/bruteforce_idx.rs:49-61, pq_idx.rs:181-191,
// 429-436) and returns it ascending.  Here every query owns a sorted list of
// k (distance,row) keys in HBM; candidates found by the scoring kernels are
// merged into it by one CTA per query with a shared-memory bitonic sort.
// Ties in distance resolve to the lower row, a deterministic order (the
// reference's order at exact ties depends on heap positions).
#include <algorithm>

#include "internal.h"
#include "select.cuh"

namespace hora {

constexpr int kMergeThreads = 512;
constexpr int kSelectThreads = 256;

// Ascending bitonic sort of P (a power of two, <= 512) keys in shared memory
// by one warp: no block barriers, so the CTA's other warps are free.
__device__ __forceinline__ void warp_bitonic_sort(uint64_t *sk, int P) {
  const int lane = threadIdx.x & 31;
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < (P >> 1); i += 32) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool asc = (lo & size) == 0;
        const uint64_t a = sk[lo], b = sk[hi];
        if ((a > b) == asc) {
          sk[lo] = b;
          sk[hi] = a;
        }
      }
      __syncwarp();
    }
  }
}

__device__ __forceinline__ void block_bitonic_sort(uint64_t *sk, int P) {
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
        int lo = 2 * i - (i & (stride - 1));
        int hi = lo + stride;
        bool asc = (lo & size) == 0;
        uint64_t a = sk[lo], b = sk[hi];
        if ((a > b) == asc) {
          sk[lo] = b;
          sk[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

// Exclusive block scan of one int per thread (blockDim.x <= 1024).
__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;
  }
  __syncthreads();
  int base = wid ? warp_sums[wid - 1] : 0;
  *total = warp_sums[nw - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void __launch_bounds__(kMergeThreads) merge_topk_kernel(
    uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap, int dense_n,
    const int *qlist, uint8_t *ovf_flag, uint32_t *ovf_counter) {
  extern __shared__ uint64_t sk[];
  __shared__ int warp_sums[32];
  const int64_t q = qlist ? qlist[blockIdx.x] : blockIdx.x;
  uint32_t c = dense_n > 0 ? (uint32_t)dense_n : count[q];
  if (c == 0) return;
  const bool ovf = c > (uint32_t)cap;
  if (ovf) c = cap;
  const int total = (int)c + k;
  int P = 1;
  while (P < total) P <<= 1;
  const uint64_t *cq = cand + q * cap;
  uint64_t *bq = best + q * k;
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    sk[i] = i < (int)c ? cq[i] : (i < total ? bq[i - c] : kEmptyKey);
  __syncthreads();
  block_bitonic_sort(sk, P);
  // keep the first occurrence of each key (a row can be offered twice when a
  // scan is repeated after a capacity overflow), compact the first k
  const int per = (P + blockDim.x - 1) / blockDim.x;
  const int beg = threadIdx.x * per, end = min(P, beg + per);
  int mine = 0;
  for (int i = beg; i < end; ++i) mine += (sk[i] != kEmptyKey && (i == 0 || sk[i] != sk[i - 1]));
  int tot;
  int pos = block_exclusive_scan(mine, warp_sums, &tot);
  for (int i = beg; i < end && pos < k; ++i) {
    if (sk[i] != kEmptyKey && (i == 0 || sk[i] != sk[i - 1])) {
      bq[pos] = sk[i];
      ++pos;
    }
  }
  for (int i = tot + threadIdx.x; i < k; i += blockDim.x) bq[i] = kEmptyKey;
  if (threadIdx.x == 0) {
    if (dense_n <= 0) count[q] = 0;
    if (ovf) {
      ovf_flag[q] = 1;
      atomicAdd(ovf_counter, 1u);
    }
  }
}

// Merge without duplicates (candidate rows are disjoint from the rows already
// in the list: chunks and lists never overlap): radix-select the k-th
// smallest of the c + k keys, gather the k winners and sort only those.
// Digits of 11/11/10 bits from the top of the 64-bit key (distance bits
// first, then the row), histogram updates aggregated per warp; the select
// stops as soon as the digit holding the k-th key holds exactly the keys
// still needed (usually once the distance bits are resolved).
__global__ void __launch_bounds__(kSelectThreads) merge_select_kernel(
    uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap, int dense_n,
    uint8_t *ovf_flag, uint32_t *ovf_counter, int sorted) {
  extern __shared__ uint64_t sk[];
  __shared__ uint32_t hist[kSelBins];
  __shared__ int sc[8];  // [0] live, [1] digit, [2] below, [3] taken, [4] remaining, [5] at digit
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t q = blockIdx.x;
  uint32_t c = dense_n > 0 ? (uint32_t)dense_n : count[q];
  if (c == 0) return;
  const bool ovf = c > (uint32_t)cap;
  if (ovf) c = cap;
  const uint64_t *cq = cand + q * cap;
  uint64_t *bq = best + q * k;
  // live keys: candidates, then the list's non-empty prefix
  const int n = (int)c + k;
  if (threadIdx.x == 0) {
    sc[0] = 0;
    sc[3] = 0;
  }
  for (int b = threadIdx.x; b < kSelBins; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  int live = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const uint64_t v = i < (int)c ? cq[i] : bq[i - c];
    sk[i] = v;
    live += v != kEmptyKey;
  }
  live = __reduce_add_sync(0xffffffffu, live);
  if (lane == 0) atomicAdd(&sc[0], live);
  __syncthreads();
  const int nl = sc[0];
  const int want = nl < k ? nl : k;
  uint64_t *sel = sk + n;  // want keys
  if (want > 0) {
    uint64_t prefix = 0, mask = 0;
    int rem = want;
    for (int pass = 0; pass < 6; ++pass) {
      const int shift = pass == 0 ? 53 : pass == 1 ? 42 : pass == 2 ? 32 : pass == 3 ? 21 : pass == 4 ? 10 : 0;
      const uint32_t dmask = (pass == 2 || pass == 5) ? 1023u : 2047u;
      for (int i0 = 0; i0 < n; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        const uint64_t v = i < n ? sk[i] : kEmptyKey;
        const bool p = v != kEmptyKey && (v & mask) == prefix;
        const unsigned pm = __ballot_sync(0xffffffffu, p);
        if (p) {
          const uint32_t dig = (uint32_t)(v >> shift) & dmask;
          const unsigned peers = __match_any_sync(pm, dig);
          if (lane == __ffs(peers) - 1) atomicAdd(&hist[dig], (uint32_t)__popc(peers));
        }
      }
      __syncthreads();
      if (warp == 0) {
        warp_find_bin(hist, (int)dmask + 1, (uint32_t)rem, sc + 1);
        __syncwarp();
        const int at = (int)hist[sc[1]];
        const int below = sc[2];
        __syncwarp();
        for (int b = lane; b <= (int)dmask; b += 32) hist[b] = 0;
        if (lane == 0) {
          sc[4] = rem - below;
          sc[5] = at;
        }
      }
      __syncthreads();
      rem = sc[4];
      prefix |= (uint64_t)sc[1] << shift;
      mask |= (uint64_t)dmask << shift;
      if (sc[5] == rem) break;  // every key under this prefix is taken
    }
    // the winners: keys whose masked top bits are <= the prefix
    for (int i0 = 0; i0 < n; i0 += blockDim.x) {
      const int i = i0 + threadIdx.x;
      const uint64_t v = i < n ? sk[i] : kEmptyKey;
      const bool p = v != kEmptyKey && (v & mask) <= prefix;
      const unsigned pm = __ballot_sync(0xffffffffu, p);
      if (pm) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&sc[3], __popc(pm));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int slot = base + __popc(pm & ((1u << lane) - 1u));
        if (p && slot < want) sel[slot] = v;  // (keys are distinct: exactly want pass)
      }
    }
    __syncthreads();
    if (sorted) {
      int P = 1;
      while (P < want) P <<= 1;
      for (int i = want + threadIdx.x; i < P; i += blockDim.x) sel[i] = kEmptyKey;
      __syncthreads();
      if (P <= 512) {
        if (warp == 0) warp_bitonic_sort(sel, P);
        __syncthreads();
      } else {
        block_bitonic_sort(sel, P);
      }
    } else if (warp == 0) {
      // unordered winners: only the largest must sit last (it is the
      // scan's threshold); keys are distinct, so one position holds it
      uint64_t mx = 0;
      int at = 0;
      for (int i = lane; i < want; i += 32)
        if (sel[i] >= mx) {
          mx = sel[i];
          at = i;
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const uint64_t m2 = __shfl_xor_sync(0xffffffffu, mx, o);
        const int a2 = __shfl_xor_sync(0xffffffffu, at, o);
        if (m2 > mx) {
          mx = m2;
          at = a2;
        }
      }
      if (lane == 0 && at != want - 1) {
        const uint64_t t = sel[want - 1];
        sel[want - 1] = mx;
        sel[at] = t;
      }
      __syncwarp();
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < k; i += blockDim.x) bq[i] = i < want ? sel[i] : kEmptyKey;
  if (threadIdx.x == 0) {
    if (dense_n <= 0) count[q] = 0;
    if (ovf) {
      ovf_flag[q] = 1;
      atomicAdd(ovf_counter, 1u);
    }
  }
}

// The same merge with one warp per query for k <= 256.  Every key (list +
// candidates) is read once; for up to 32 x kWmRegs keys the warp keeps their
// high (distance) words in registers, 40 per lane.  The radix select runs on
// key - kmin, kmin = the smallest high word (low word zero), with its first
// 8-bit digit at the top of the key range, so the leading bits that every key
// shares cost no pass and the keys spread over the bins (plain shared
// atomics, few collisions).  While the selection stays within the distance
// word it runs on the registers alone, and only the winners' full keys are
// read again; a selection that needs the row bits (ties), or a larger key
// set, reads the keys from global memory on each pass.  The winners are
// sorted only for a final list; an intermediate list (sorted = false) only
// needs its largest key at k - 1, where the candidate filter reads the
// threshold.  No block barrier anywhere.
constexpr int kWmWarps = 8, kWmMaxK = 256, kWmRegs = 40;

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  return v;
}

template <bool SORTED>
__global__ void __launch_bounds__(kWmWarps * 32, 3) merge_warp_kernel(
    uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap, int dense_n, const int *qlist,
    int64_t nq, uint8_t *ovf_flag, uint32_t *ovf_counter) {
  __shared__ uint32_t hist_all[kWmWarps][256];
  __shared__ uint64_t sel_all[kWmWarps][kWmMaxK];
  __shared__ int dig_all[kWmWarps][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t qi = (int64_t)blockIdx.x * kWmWarps + warp;
  if (qi >= nq) return;
  const int64_t q = qlist ? qlist[qi] : qi;
  uint32_t *hist = hist_all[warp];
  uint64_t *sel = sel_all[warp];
  int *dig = dig_all[warp];
  uint32_t c = dense_n > 0 ? (uint32_t)dense_n : count[q];
  if (c == 0) return;
  const bool ovf = c > (uint32_t)cap;
  if (ovf) c = cap;
  const uint64_t *cq = cand + q * cap;
  uint64_t *bq = best + q * k;
  const int n = (int)c + k;
  auto key_at = [&](int i) -> uint64_t { return i < (int)c ? cq[i] : bq[i - c]; };
  const bool inreg = n <= 32 * kWmRegs;
  const int nm = (n + 31) >> 5;  // register slots in use (uniform in the warp)

  // one read of every key: live count and the range of the high words (no
  // live key has the empty key's high word 0xffffffff, which is the largest)
  uint32_t hw[kWmRegs];
  int live = 0;
  uint32_t hmin = 0xffffffffu, hmax = 0;
  if (inreg) {
#pragma unroll
    for (int b = 0; b < kWmRegs; b += 8) {
      if (b >= nm) break;
      uint64_t v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = (b + u) * 32 + lane;
        v[u] = i < n ? key_at(i) : kEmptyKey;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) hw[b + u] = (uint32_t)(v[u] >> 32);
    }
#pragma unroll
    for (int m = 0; m < kWmRegs; ++m) {
      if (m >= nm) break;
      const bool ok = hw[m] != 0xffffffffu;
      live += ok;
      hmin = min(hmin, hw[m]);
      hmax = max(hmax, ok ? hw[m] : 0u);
    }
  } else {
    for (int i = lane; i < n; i += 32) {
      const uint32_t hi = (uint32_t)(key_at(i) >> 32);
      const bool ok = hi != 0xffffffffu;
      live += ok;
      hmin = min(hmin, hi);
      hmax = max(hmax, ok ? hi : 0u);
    }
  }
  live = __reduce_add_sync(0xffffffffu, live);
  hmin = __reduce_min_sync(0xffffffffu, hmin);
  hmax = __reduce_max_sync(0xffffffffu, hmax);
  // every live key lies in [kmin, kmax]; key - kmin keeps the low word and
  // subtracts hmin from the high one
  const uint64_t kmin = (uint64_t)hmin << 32, kmax = ((uint64_t)hmax << 32) | 0xffffffffull;
  const int want = live < k ? live : k;
  // the winners are the live keys with key - kmin <= bound
  uint64_t bound = kmax - kmin;
  if (want > 0 && want < live) {
    const uint64_t span = kmax - kmin;
    int shift = 64 - __clzll((long long)span) - 8;
    shift = shift < 0 ? 0 : shift;
    uint64_t prefix = 0, mask = 0;
    int rem = want;
    for (;;) {
      for (int b = lane; b < 256; b += 32) hist[b] = 0;
      __syncwarp();
      if (shift >= 32) {
        // the digit and every fixed bit lie in the high word
        const uint32_t mh = (uint32_t)(mask >> 32), ph = (uint32_t)(prefix >> 32);
        const int sh = shift - 32;
        if (inreg) {
#pragma unroll
          for (int m = 0; m < kWmRegs; ++m) {
            if (m >= nm) break;
            const uint32_t dh = hw[m] - hmin;
            if (hw[m] != 0xffffffffu && (dh & mh) == ph) atomicAdd(&hist[(dh >> sh) & 255u], 1u);
          }
        } else {
#pragma unroll 4
          for (int i = lane; i < n; i += 32) {
            const uint32_t hi = (uint32_t)(key_at(i) >> 32);
            const uint32_t dh = hi - hmin;
            if (hi != 0xffffffffu && (dh & mh) == ph) atomicAdd(&hist[(dh >> sh) & 255u], 1u);
          }
        }
      } else {
#pragma unroll 4
        for (int i = lane; i < n; i += 32) {
          const uint64_t v = key_at(i);
          const uint64_t d = v - kmin;
          if (v != kEmptyKey && (d & mask) == prefix) atomicAdd(&hist[(uint32_t)(d >> shift) & 255u], 1u);
        }
      }
      __syncwarp();
      warp_find_digit(hist, (uint32_t)rem, dig);
      __syncwarp();
      const int dd = dig[0], at = (int)hist[dd];
      rem -= dig[1];
      prefix |= (uint64_t)dd << shift;
      mask |= (uint64_t)0xff << shift;
      __syncwarp();
      if (at == rem || shift == 0) break;  // every key under this prefix is taken
      shift = shift >= 8 ? shift - 8 : 0;
    }
    // the largest d under the prefix (d has no bits above the first digit)
    bound = prefix | ((1ull << shift) - 1ull);
  }
  if (want > 0) {
    int taken = 0;
    const unsigned below = (1u << lane) - 1u;
    if (inreg && (uint32_t)bound == 0xffffffffu) {
      // the test needs the high words only: d <= bound iff hi - hmin <= bound's high word
      const uint32_t bh = (uint32_t)(bound >> 32);
#pragma unroll
      for (int m = 0; m < kWmRegs; ++m) {
        if (m >= nm) break;
        const bool p = hw[m] != 0xffffffffu && hw[m] - hmin <= bh;
        const unsigned pm = __ballot_sync(0xffffffffu, p);
        const int slot = taken + __popc(pm & below);
        if (p && slot < want) sel[slot] = key_at(m * 32 + lane);
        taken += __popc(pm);
      }
    } else {
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        const uint64_t v = i < n ? key_at(i) : kEmptyKey;
        const bool p = v != kEmptyKey && v - kmin <= bound;
        const unsigned pm = __ballot_sync(0xffffffffu, p);
        const int slot = taken + __popc(pm & below);
        if (p && slot < want) sel[slot] = v;
        taken += __popc(pm);
      }
    }
    __syncwarp();
    if (SORTED) {
      int P = 1;
      while (P < want) P <<= 1;
      for (int i = want + lane; i < P; i += 32) sel[i] = kEmptyKey;
      __syncwarp();
      warp_bitonic_sort(sel, P);
    } else if (want == k) {
      // the largest winner to slot k - 1
      uint64_t m = 0;
      int at = -1;
      for (int i = lane; i < want; i += 32)
        if (sel[i] >= m) {
          m = sel[i];
          at = i;
        }
      const uint64_t mx = warp_max_u64(m);
      const unsigned who = __ballot_sync(0xffffffffu, m == mx && at >= 0);
      const int src = __shfl_sync(0xffffffffu, at, __ffs(who) - 1);
      if (lane == 0 && src != want - 1) {
        sel[src] = sel[want - 1];
        sel[want - 1] = mx;
      }
      __syncwarp();
    }
  }
  for (int i = lane; i < k; i += 32) bq[i] = i < want ? sel[i] : kEmptyKey;
  if (lane == 0) {
    if (dense_n <= 0) count[q] = 0;
    if (ovf) {
      ovf_flag[q] = 1;
      atomicAdd(ovf_counter, 1u);
    }
  }
}

// k in (256, 4096]: the warp kernel's scheme with one CTA of 256 threads per
// query.  Every key is read once; the distance words of up to 12,288 keys
// stay in registers (48 per thread); the radix select runs on key - kmin
// with an 11-bit first digit at the top of the key range, on the 32-bit words
// while the selection stays within them (else on the full keys, re-read);
// only the winners' full keys are read again.  Shared memory holds the
// 2,048-bin histogram and the winners (sorted for a final list; otherwise
// only the largest moves to k - 1).
constexpr int kMbThreads = 256, kMbRegs = 48, kMbMaxK = 4096;

template <bool SORTED>
__global__ void __launch_bounds__(kMbThreads, 2) merge_block_kernel(
    uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap, int dense_n, const int *qlist,
    uint8_t *ovf_flag, uint32_t *ovf_counter) {
  extern __shared__ uint64_t mb_sel[];  // P >= k winners
  __shared__ uint32_t hist[kSelBins];
  __shared__ uint32_t red[3][kMbThreads / 32];
  __shared__ int sc[8];  // [1] bin, [2] below, [3] taken, [4] remaining, [5] at bin
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t q = qlist ? qlist[blockIdx.x] : blockIdx.x;
  uint32_t c = dense_n > 0 ? (uint32_t)dense_n : count[q];
  if (c == 0) return;
  const bool ovf = c > (uint32_t)cap;
  if (ovf) c = cap;
  const uint64_t *cq = cand + q * cap;
  uint64_t *bq = best + q * k;
  const int n = (int)c + k;  // <= kMbThreads * kMbRegs: the host checks
  const int nm = (n + kMbThreads - 1) / kMbThreads;  // register slots in use (uniform)
  auto key_at = [&](int i) -> uint64_t { return i < (int)c ? cq[i] : bq[i - c]; };

  // one read of every key: the distance words, live count and range
  uint32_t hw[kMbRegs];
#pragma unroll
  for (int b = 0; b < kMbRegs; b += 8) {
    if (b >= nm) break;
    uint64_t v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = (b + u) * kMbThreads + tid;
      v[u] = i < n ? key_at(i) : kEmptyKey;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) hw[b + u] = (uint32_t)(v[u] >> 32);
  }
  int live = 0;
  uint32_t hmin = 0xffffffffu, hmax = 0;
#pragma unroll
  for (int m = 0; m < kMbRegs; ++m) {
    if (m >= nm) break;
    const bool ok = hw[m] != 0xffffffffu;
    live += ok;
    hmin = min(hmin, hw[m]);
    hmax = max(hmax, ok ? hw[m] : 0u);
  }
  live = __reduce_add_sync(0xffffffffu, live);
  hmin = __reduce_min_sync(0xffffffffu, hmin);
  hmax = __reduce_max_sync(0xffffffffu, hmax);
  if (lane == 0) {
    red[0][warp] = (uint32_t)live;
    red[1][warp] = hmin;
    red[2][warp] = hmax;
  }
  for (int b = tid; b < kSelBins; b += kMbThreads) hist[b] = 0;
  if (tid == 0) sc[3] = 0;
  __syncthreads();
  live = 0;
  hmin = 0xffffffffu;
  hmax = 0;
#pragma unroll
  for (int w = 0; w < kMbThreads / 32; ++w) {
    live += (int)red[0][w];
    hmin = min(hmin, red[1][w]);
    hmax = max(hmax, red[2][w]);
  }
  const uint64_t kmin = (uint64_t)hmin << 32, kmax = ((uint64_t)hmax << 32) | 0xffffffffull;
  const int want = live < k ? live : k;
  uint64_t bound = kmax - kmin;
  if (want > 0 && want < live) {
    const uint64_t span = kmax - kmin;
    int shift = 64 - __clzll((long long)span) - 11;
    shift = shift < 0 ? 0 : shift;
    uint64_t prefix = 0, mask = 0;
    int rem = want;
    for (;;) {
      if (shift >= 32) {
        const uint32_t mh = (uint32_t)(mask >> 32), ph = (uint32_t)(prefix >> 32);
        const int sh = shift - 32;
#pragma unroll
        for (int m = 0; m < kMbRegs; ++m) {
          if (m >= nm) break;
          const uint32_t dh = hw[m] - hmin;
          if (hw[m] != 0xffffffffu && (dh & mh) == ph) atomicAdd(&hist[(dh >> sh) & (kSelBins - 1)], 1u);
        }
      } else {
        for (int i = tid; i < n; i += kMbThreads) {
          const uint64_t v = key_at(i);
          const uint64_t d = v - kmin;
          if (v != kEmptyKey && (d & mask) == prefix)
            atomicAdd(&hist[(uint32_t)(d >> shift) & (kSelBins - 1)], 1u);
        }
      }
      __syncthreads();
      if (warp == 0) {
        warp_find_bin(hist, kSelBins, (uint32_t)rem, sc + 1);
        __syncwarp();
        if (lane == 0) {
          sc[4] = rem - sc[2];
          sc[5] = (int)hist[sc[1]];
        }
      }
      __syncthreads();
      const int dd = sc[1], at = sc[5];
      rem = sc[4];
      prefix |= (uint64_t)dd << shift;
      mask |= (uint64_t)(kSelBins - 1) << shift;
      for (int b = tid; b < kSelBins; b += kMbThreads) hist[b] = 0;
      __syncthreads();
      if (at == rem || shift == 0) break;  // every key under this prefix is taken
      shift = shift >= 11 ? shift - 11 : 0;
    }
    // the largest d under the prefix (d has no bits above the first digit)
    bound = prefix | ((1ull << shift) - 1ull);
  }
  if (want > 0) {
    const unsigned below = (1u << lane) - 1u;
    if ((uint32_t)bound == 0xffffffffu) {
      // d <= bound iff hi - hmin <= bound's high word
      const uint32_t bh = (uint32_t)(bound >> 32);
#pragma unroll
      for (int m = 0; m < kMbRegs; ++m) {
        if (m >= nm) break;
        const bool p = hw[m] != 0xffffffffu && hw[m] - hmin <= bh;
        const unsigned pm = __ballot_sync(0xffffffffu, p);
        if (pm) {
          int base = 0;
          if (lane == 0) base = atomicAdd(&sc[3], __popc(pm));
          base = __shfl_sync(0xffffffffu, base, 0);
          const int slot = base + __popc(pm & below);
          if (p && slot < want) mb_sel[slot] = key_at(m * kMbThreads + tid);
        }
      }
    } else {
      for (int i0 = 0; i0 < n; i0 += kMbThreads) {
        const int i = i0 + tid;
        const uint64_t v = i < n ? key_at(i) : kEmptyKey;
        const bool p = v != kEmptyKey && v - kmin <= bound;
        const unsigned pm = __ballot_sync(0xffffffffu, p);
        if (pm) {
          int base = 0;
          if (lane == 0) base = atomicAdd(&sc[3], __popc(pm));
          base = __shfl_sync(0xffffffffu, base, 0);
          const int slot = base + __popc(pm & below);
          if (p && slot < want) mb_sel[slot] = v;
        }
      }
    }
    __syncthreads();
    if (SORTED) {
      int P = 1;
      while (P < want) P <<= 1;
      for (int i = want + tid; i < P; i += kMbThreads) mb_sel[i] = kEmptyKey;
      __syncthreads();
      block_bitonic_sort(mb_sel, P);
    } else if (want == k && warp == 0) {
      // the largest winner to slot k - 1
      uint64_t m = 0;
      int at = -1;
      for (int i = lane; i < want; i += 32)
        if (mb_sel[i] >= m) {
          m = mb_sel[i];
          at = i;
        }
      const uint64_t mx = warp_max_u64(m);
      const unsigned who = __ballot_sync(0xffffffffu, m == mx && at >= 0);
      const int src = __shfl_sync(0xffffffffu, at, __ffs(who) - 1);
      if (lane == 0 && src != want - 1) {
        mb_sel[src] = mb_sel[want - 1];
        mb_sel[want - 1] = mx;
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < k; i += kMbThreads) bq[i] = i < want ? mb_sel[i] : kEmptyKey;
  if (tid == 0) {
    if (dense_n <= 0) count[q] = 0;
    if (ovf) {
      ovf_flag[q] = 1;
      atomicAdd(ovf_counter, 1u);
    }
  }
}

int merge_smem_bytes(int k, int cap) {
  int P = 1;
  while (P < k + cap) P <<= 1;
  return P * 8;
}

int launch_merge_topk(uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap,
                      int dense_n, const int *qlist, int64_t nlist, uint8_t *ovf_flag,
                      uint32_t *ovf_counter, cudaStream_t s, bool sorted, bool disjoint) {
  if (nlist <= 0) return HORA_OK;
  HORA_SMEM_ATTR(merge_topk_kernel, 200 * 1024);
  HORA_SMEM_ATTR(merge_select_kernel, 200 * 1024);
  const int cmax = dense_n > 0 ? dense_n : cap;
  // a query list takes the radix merges only for candidates disjoint from
  // the list (the rescans after an overflow re-offer rows: they deduplicate)
  const bool radix = !qlist || disjoint;
  if (radix && k <= kWmMaxK) {
    ProfScope ps("topk_merge", s);
    const unsigned grid = (unsigned)ceil_div(nlist, (int64_t)kWmWarps);
    if (sorted)
      merge_warp_kernel<true><<<grid, kWmWarps * 32, 0, s>>>(best, k, cand, count, cap, dense_n, qlist, nlist,
                                                                 ovf_flag, ovf_counter);
    else
      merge_warp_kernel<false><<<grid, kWmWarps * 32, 0, s>>>(best, k, cand, count, cap, dense_n, qlist, nlist,
                                                                  ovf_flag, ovf_counter);
    HORA_LAUNCHED();
    return HORA_OK;
  }
  if (radix && k <= kMbMaxK && cmax + k <= kMbThreads * kMbRegs) {
    int P = 1;
    while (P < k) P <<= 1;
    const int smem = P * 8;
    HORA_SMEM_ATTR(merge_block_kernel<true>, smem);
    HORA_SMEM_ATTR(merge_block_kernel<false>, smem);
    ProfScope ps("topk_merge", s);
    if (sorted)
      merge_block_kernel<true><<<(unsigned)nlist, kMbThreads, smem, s>>>(best, k, cand, count, cap, dense_n,
                                                                      qlist, ovf_flag, ovf_counter);
    else
      merge_block_kernel<false><<<(unsigned)nlist, kMbThreads, smem, s>>>(best, k, cand, count, cap, dense_n,
                                                                       qlist, ovf_flag, ovf_counter);
    HORA_LAUNCHED();
    return HORA_OK;
  }
  if (!qlist) {
    int P = 1;
    while (P < k) P <<= 1;
    const size_t smem = (size_t)(cmax + k + P) * 8;
    if (smem <= 200 * 1024) {
      ProfScope ps("topk_merge", s);
      merge_select_kernel<<<(unsigned)nlist, kSelectThreads, smem, s>>>(best, k, cand, count, cap, dense_n,
                                                                       ovf_flag, ovf_counter, sorted ? 1 : 0);
      HORA_LAUNCHED();
      return HORA_OK;
    }
  }
  int smem = merge_smem_bytes(k, cmax);
  if (smem > 200 * 1024) return fail(HORA_ECAP, "merge: k + candidate capacity too large");
  ProfScope ps("topk_merge", s);
  merge_topk_kernel<<<(unsigned)nlist, kMergeThreads, smem, s>>>(best, k, cand, count, cap, dense_n,
                                                                qlist, ovf_flag, ovf_counter);
  HORA_LAUNCHED();
  return HORA_OK;
}

__global__ void keys_to_results_kernel(const uint64_t *keys, int64_t n, const uint64_t *idt,
                                       uint64_t *ids, float *dist) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = keys[i];
  if (k == kEmptyKey) {
    if (ids) ids[i] = HORA_NO_ID;
    if (dist) dist[i] = __int_as_float(0x7f800000);
  } else {
    if (ids) ids[i] = idt ? idt[key_row(k)] : key_row(k);
    if (dist) dist[i] = key_dist(k);
  }
}

int launch_keys_to_results(const uint64_t *keys, int64_t n, const uint64_t *idt, uint64_t *ids,
                           float *dist, cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  ProfScope ps("keys_to_results", s);
  keys_to_results_kernel<<<ceil_div(n, 256), 256, 0, s>>>(keys, n, idt, ids, dist);
  HORA_LAUNCHED();
  return HORA_OK;
}

__global__ void gather_rows_kernel(const uint64_t *keys, int64_t n, const float *base, int64_t ld,
                                   int64_t dim, float *out) {
  int64_t r = blockIdx.x;
  uint64_t k = keys[r];
  for (int64_t t = threadIdx.x; t < dim; t += blockDim.x)
    out[r * dim + t] = k == kEmptyKey ? 0.0f : base[(int64_t)key_row(k) * ld + t];
}

int launch_gather_rows(const uint64_t *keys, int64_t n, const float *base, int64_t ld,
                       int64_t dim, float *out, cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  gather_rows_kernel<<<(unsigned)n, 128, 0, s>>>(keys, n, base, ld, dim, out);
  HORA_LAUNCHED();
  return HORA_OK;
}

__global__ void __launch_bounds__(kMergeThreads) rows_topk_kernel(const float *D, int64_t cols,
                                                                  int64_t ldd, int k, int P,
                                                                  uint64_t *out) {
  extern __shared__ uint64_t sk[];
  const int64_t r = blockIdx.x;
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    sk[i] = i < cols ? make_key(D[r * ldd + i], (uint32_t)i) : kEmptyKey;
  __syncthreads();
  block_bitonic_sort(sk, P);
  for (int i = threadIdx.x; i < k; i += blockDim.x) out[r * k + i] = sk[i];
}

// The k smallest (distance, column) keys of each row, ascending, for rows of
// up to 32 x kWmRegs columns and k <= 256: one warp per row, the merge
// kernel's scheme with every key in registers (the distance word, and the
// column implied by the register's place), one read of the row, a radix
// select from the top of the row's key range and a warp sort of the winners.
__global__ void __launch_bounds__(kWmWarps * 32) rows_select_warp_kernel(const float *D, int64_t rows,
                                                                        int cols, int64_t ldd, int k,
                                                                        uint64_t *out) {
  __shared__ uint32_t hist_all[kWmWarps][256];
  __shared__ uint64_t sel_all[kWmWarps][kWmMaxK];
  __shared__ int dig_all[kWmWarps][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r = (int64_t)blockIdx.x * kWmWarps + warp;
  if (r >= rows) return;
  uint32_t *hist = hist_all[warp];
  uint64_t *sel = sel_all[warp];
  int *dig = dig_all[warp];
  const int nm = (cols + 31) >> 5;  // register slots in use (uniform)
  uint32_t hw[kWmRegs];
#pragma unroll
  for (int m = 0; m < kWmRegs; ++m) {
    if (m >= nm) break;
    const int i = m * 32 + lane;
    hw[m] = i < cols ? f2ord(D[r * ldd + i]) : 0xffffffffu;
  }
  int live = 0;
  uint32_t hmin = 0xffffffffu, hmax = 0;
#pragma unroll
  for (int m = 0; m < kWmRegs; ++m) {
    if (m >= nm) break;
    const bool ok = hw[m] != 0xffffffffu;
    live += ok;
    hmin = min(hmin, hw[m]);
    hmax = max(hmax, ok ? hw[m] : 0u);
  }
  live = __reduce_add_sync(0xffffffffu, live);
  hmin = __reduce_min_sync(0xffffffffu, hmin);
  hmax = __reduce_max_sync(0xffffffffu, hmax);
  const uint64_t kmin = (uint64_t)hmin << 32, kmax = ((uint64_t)hmax << 32) | 0xffffffffull;
  const int want = live < k ? live : k;
  uint64_t bound = kmax - kmin;
  if (want > 0 && want < live) {
    const uint64_t span = kmax - kmin;
    int shift = 64 - __clzll((long long)span) - 8;
    shift = shift < 0 ? 0 : shift;
    uint64_t prefix = 0, mask = 0;
    int rem = want;
    for (;;) {
      for (int b = lane; b < 256; b += 32) hist[b] = 0;
      __syncwarp();
      if (shift >= 32) {
        const uint32_t mh = (uint32_t)(mask >> 32), ph = (uint32_t)(prefix >> 32);
        const int sh = shift - 32;
#pragma unroll
        for (int m = 0; m < kWmRegs; ++m) {
          if (m >= nm) break;
          const uint32_t dh = hw[m] - hmin;
          if (hw[m] != 0xffffffffu && (dh & mh) == ph) atomicAdd(&hist[(dh >> sh) & 255u], 1u);
        }
      } else {
#pragma unroll
        for (int m = 0; m < kWmRegs; ++m) {
          if (m >= nm) break;
          const uint64_t d = ((((uint64_t)hw[m]) << 32) | (uint32_t)(m * 32 + lane)) - kmin;
          if (hw[m] != 0xffffffffu && (d & mask) == prefix) atomicAdd(&hist[(uint32_t)(d >> shift) & 255u], 1u);
        }
      }
      __syncwarp();
      warp_find_digit(hist, (uint32_t)rem, dig);
      __syncwarp();
      const int dd = dig[0], at = (int)hist[dd];
      rem -= dig[1];
      prefix |= (uint64_t)dd << shift;
      mask |= (uint64_t)0xff << shift;
      __syncwarp();
      if (at == rem || shift == 0) break;
      shift = shift >= 8 ? shift - 8 : 0;
    }
    bound = prefix | ((1ull << shift) - 1ull);
  }
  if (want > 0) {
    int taken = 0;
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int m = 0; m < kWmRegs; ++m) {
      if (m >= nm) break;
      const uint64_t key = (((uint64_t)hw[m]) << 32) | (uint32_t)(m * 32 + lane);
      const bool p = hw[m] != 0xffffffffu && key - kmin <= bound;
      const unsigned pm = __ballot_sync(0xffffffffu, p);
      const int slot = taken + __popc(pm & below);
      if (p && slot < want) sel[slot] = key;
      taken += __popc(pm);
    }
    int P = 1;
    while (P < want) P <<= 1;
    __syncwarp();
    for (int i = want + lane; i < P; i += 32) sel[i] = kEmptyKey;
    __syncwarp();
    warp_bitonic_sort(sel, P);
  }
  for (int i = lane; i < k; i += 32) out[r * k + i] = i < want ? sel[i] : kEmptyKey;
}

// Small k (<= K): one warp per row; each lane keeps the K smallest keys
// (ordered distance bits << 32 | column) of its columns (lane, lane + 32,
// ...: coalesced reads of any row length) in registers, sorted by insertion;
// then k rounds of a warp minimum over the lanes' heads, the owner popping
// its head, write the k smallest keys in ascending order.
template <int K>
__global__ void __launch_bounds__(256) rows_topk_small_kernel(const float *D, int64_t rows, int64_t cols,
                                                              int64_t ldd, int k, uint64_t *out) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= rows) return;
  uint64_t best[K];
#pragma unroll
  for (int i = 0; i < K; ++i) best[i] = kEmptyKey;
  for (int64_t c = lane; c < cols; c += 32) {
    uint64_t key = ((uint64_t)f2ord(D[r * ldd + c]) << 32) | (uint32_t)c;
    if (key < best[K - 1]) {
#pragma unroll
      for (int i = 0; i < K; ++i) {
        const uint64_t lo = key < best[i] ? key : best[i], hi = key < best[i] ? best[i] : key;
        best[i] = lo;
        key = hi;
      }
    }
  }
  for (int j = 0; j < k; ++j) {
    uint64_t m = best[0];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const uint64_t y = __shfl_xor_sync(0xffffffffu, m, o);
      m = y < m ? y : m;
    }
    if (lane == 0) out[r * k + j] = m;
    if (m != kEmptyKey && best[0] == m) {  // keys are distinct: one owner
#pragma unroll
      for (int i = 0; i < K - 1; ++i) best[i] = best[i + 1];
      best[K - 1] = kEmptyKey;
    }
  }
}

int launch_rows_topk(const float *D, int64_t rows, int64_t cols, int64_t ldd, int k,
                     uint64_t *out, cudaStream_t s) {
  if (rows <= 0) return HORA_OK;
  if (k <= 16) {
    ProfScope ps("rows_topk", s);
    const unsigned g = (unsigned)ceil_div(rows, (int64_t)8);
    if (k <= 2)
      rows_topk_small_kernel<2><<<g, 256, 0, s>>>(D, rows, cols, ldd, k, out);
    else if (k <= 4)
      rows_topk_small_kernel<4><<<g, 256, 0, s>>>(D, rows, cols, ldd, k, out);
    else if (k <= 8)
      rows_topk_small_kernel<8><<<g, 256, 0, s>>>(D, rows, cols, ldd, k, out);
    else
      rows_topk_small_kernel<16><<<g, 256, 0, s>>>(D, rows, cols, ldd, k, out);
    HORA_LAUNCHED();
    return HORA_OK;
  }
  if (k <= kWmMaxK && cols <= 32 * kWmRegs) {
    ProfScope ps("rows_topk", s);
    rows_select_warp_kernel<<<(unsigned)ceil_div(rows, (int64_t)kWmWarps), kWmWarps * 32, 0, s>>>(
        D, rows, (int)cols, ldd, k, out);
    HORA_LAUNCHED();
    return HORA_OK;
  }
  int P = 1;
  while (P < cols || P < k) P <<= 1;
  if (P * 8 > 200 * 1024) return fail(HORA_ECAP, "rows_topk: too many columns");
  HORA_SMEM_ATTR(rows_topk_kernel, 200 * 1024);
  ProfScope ps("rows_topk", s);
  rows_topk_kernel<<<(unsigned)rows, kMergeThreads, P * 8, s>>>(D, cols, ldd, k, P, out);
  HORA_LAUNCHED();
  return HORA_OK;
}

}  // namespace hora
