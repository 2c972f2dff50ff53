// bf_lowp.cu — brute-force scoring on the 5th-generation tensor cores
// (tcgen05.mma, TMA, TMEM) in BF16 or FP8 e4m3 with FP32 accumulation,
// followed by an exact FP32 rerank of a widened candidate list.
//
// Scoring (not in the reference; it replaces the per-row metric calls of
// BruteForceIndex::node_search_k, src/index/bruteforce_idx.rs:49-61, for the
// approximate first pass):
//   Euclidean         d~ = |q|^2 + |x|^2 - 2 <q~, x~>   (norms exact, from FP64)
//   DotProduct        d~ = <q~, x~>
//   CosineSimilarity  d~ = -<q~, x~> / (|q| |x|)
// with q~, x~ the BF16 (or scaled e4m3) copies.  Each query keeps its R best
// approximate keys through the same chunked candidate scan as the exact path;
// the R rows are then rescored exactly in FP32 in the reference's op order
// and the k best returned, so every returned distance is exact.  Manhattan
// has no tensor-core form and always runs exactly on the CUDA cores.
//
// Kernel layout: CTA = 18 warps over 128 queries x 4,096 rows.  Warp 0
// issues TMA loads (the query tile once, then a ring of 256-row base tiles),
// warp 1 owns TMEM (2 accumulator buffers of 256 columns) and issues one
// 128 x 256 tcgen05.mma per K step (a 256-wide N reads the query operand from
// shared memory once per 256 rows), warps 2-17 drain the accumulators with
// tcgen05.ld (one query row per TMEM lane, two 32-column slices per warp; the
// buffer is released once the last slice is in registers), test a slice's
// extreme against the query's current R-th key and, on a hit, stage the keys
// in shared memory (flushed to the query's list 8 at a time, one atomic per
// flush).  Every mbarrier wait is bounded; a CTA that gives up raises an
// error flag read by the host, waits for its MMAs and frees TMEM.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cfloat>
#include <cstring>

#include "dist_tile.cuh"
#include "index.h"
#include "tc_ptx.cuh"

namespace hora {

constexpr int kLpBM = 128;           // queries per CTA (TMEM lanes)
constexpr int kLpBN = 256;           // base rows per tile (accumulator columns, MMA N)
constexpr int kLpNB = 2;             // TMEM accumulator buffers (2 x 256 columns)
constexpr int kLpThreads = 576;      // 18 warps
constexpr int kLpEpiThreads = 512;   // warps 2..17
// Base tiles per CTA: 32 (8,192 rows) amortises the CTA prologue (measured
// best of 16-64 at 10k queries); a launch with few query blocks takes 16 or
// 8 so that it still spreads over every SM (see lp_tiles_per_cta).
constexpr int kLpTilesPerCta = 32;
constexpr int kLpMinTilesPerCta = 8;
constexpr int kLpSlices = kLpBN / 4 / 32;  // 32-column slices per drain warp and tile
constexpr int kLpMaxStages = 8;
constexpr int kLpBarSlots = 48;  // u64 slots for the barriers, TMEM address and abort flag
// Filter-mode hits are staged per drain thread in shared memory and
// appended to the query's global list kLpHitBuf at a time (one atomic per
// flush instead of one per hit, off the per-tile critical path).
constexpr int kLpHitBuf = 8;
constexpr int kLpHitBytes = kLpHitBuf * kLpEpiThreads * 8;

// The low-precision base is kept as the shared-memory image of each 256-row
// base tile, tile after tile: its K blocks (256 rows x 128 bytes each, the
// 16-byte chunks of row r permuted by chunk ^ (r % 8): the 128-byte swizzle
// the MMA descriptors read), then for BF16 Euclidean the two 8-column halves
// of the norm block (256 rows x 16 bytes each, unswizzled).  One bulk copy
// moves a whole tile into a ring stage; rows past n are zero.
struct LowpState {
  int prec = 0, metric = 0;
  int64_t n = 0, Dp = 0;
  DevBuf tiles;    // ceil(n / 256) x tile_bytes
  int64_t tile_bytes = 0;
  DevBuf xsq;      // n f32 exact squared norms
  DevBuf xscale;   // n f32 (e4m3 per-row scale)
  // BF16 Euclidean on at least kProbeMinRows rows: pivot clusters of the base
  // (see ensure_pivots), built on first use
  int pc = 0;      // pivots (0: not built)
  DevBuf centers;  // pc x ld f32
  DevBuf coff;     // pc + 1 int64 member offsets
  DevBuf cmem;     // n uint32 member rows, cluster after cluster, ascending
  DevBuf xsqmax;   // 1 f32: the largest squared row norm
  DevBuf ctiles;   // the pivots' BF16 tile image (the BF16 base's layout, also for an FP8 base)
  int64_t ctile_bytes = 0;
  int cnkb = 0;    // the pivot image's 128-byte K blocks
  // BF16 Euclidean: the largest |x - bf16(x)| over the rows (1 f32, rounded
  // up), the rows' share of the certified exact search's error bound
  DevBuf dxmax;
};

void lowp_state_free(LowpState *p) { delete p; }

struct LpParams {
  int64_t nq;
  const int *qmap;
  const uint8_t *tiles;  // the base's tile image (see LowpState)
  int64_t r_begin, r_end;
  int nkb;        // 128-byte K blocks per row (1 or 2)
  int stages;     // base-tile ring depth
  const float *xsq, *xscale, *xnorm;
  const float *qsq, *qscale, *qnorm;
  uint64_t *best;
  int k;
  uint64_t *cand;
  int cap;
  uint32_t *count;
  int *err;
  int dense_hits;  // hit-dense launch: the warp-converged staging (stage_hits)
  int tpc;         // base tiles per CTA (lp_tiles_per_cta)
  const float *tau0;  // per query starting distance threshold (filter mode), or null
};

// BF16 Euclidean folds the row norm into the MMA: one extra K = 16 step
// whose A columns are (1, 1, 1, 0...) and whose B columns hold -|x|^2 / 2
// split into three BF16 parts, so the accumulator is <q,x> - |x|^2/2 and the
// drain needs one compare per column.  Those 16-column blocks use the
// unswizzled K-major layout: 8-row x 16-byte core matrices, 128 bytes apart
// along M/N, the two 8-column halves kNormHalfA / kNormHalfB bytes apart.
constexpr uint32_t kNormHalfA = kLpBM * 16, kNormHalfB = kLpBN * 16;
constexpr uint32_t kNormBytesA = 2 * kNormHalfA, kNormBytesB = 2 * kNormHalfB;

// What the drain needs to test and append the columns that hit.
struct DrainCtx {
  uint64_t *cand;
  uint32_t *count;
  uint64_t *hb;  // this thread's staging column (stride kLpEpiThreads)
  int64_t qid, rt, r_begin, r_end;
  int cap;
  float qa, tau_d;  // the query's current R-th key (distance, row)
  uint32_t tau_r;
};

// Three-input max / min (PTX max.f32 / min.f32 with three sources): the
// slice extreme in 17 operations instead of 31.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// The largest (MIN_: smallest) of the 32 accumulators of a slice.
template <bool MIN_>
__device__ __forceinline__ float slice_extreme(const uint32_t (&v)[32]) {
  float e[11];
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const float a = __uint_as_float(v[3 * i]), b = __uint_as_float(v[3 * i + 1]), c = __uint_as_float(v[3 * i + 2]);
    e[i] = MIN_ ? min3f(a, b, c) : max3f(a, b, c);
  }
  e[10] = MIN_ ? fminf(__uint_as_float(v[30]), __uint_as_float(v[31]))
               : fmaxf(__uint_as_float(v[30]), __uint_as_float(v[31]));
  const float f0 = MIN_ ? min3f(e[0], e[1], e[2]) : max3f(e[0], e[1], e[2]);
  const float f1 = MIN_ ? min3f(e[3], e[4], e[5]) : max3f(e[3], e[4], e[5]);
  const float f2 = MIN_ ? min3f(e[6], e[7], e[8]) : max3f(e[6], e[7], e[8]);
  const float f3 = MIN_ ? fminf(e[9], e[10]) : fmaxf(e[9], e[10]);
  const float g = MIN_ ? min3f(f0, f1, f2) : max3f(f0, f1, f2);
  return MIN_ ? fminf(g, f3) : fmaxf(g, f3);
}

// v[j] for a lane-dependent j without local memory: a 5-level select tree
// over the 32 accumulator registers (31 selects, rare path only).
__device__ __forceinline__ uint32_t pick32(const uint32_t (&v)[32], int j) {
  uint32_t a[16], b[8], c[4];
#pragma unroll
  for (int i = 0; i < 16; ++i) a[i] = (j & 16) ? v[i + 16] : v[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) b[i] = (j & 8) ? a[i + 8] : a[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) c[i] = (j & 4) ? b[i + 4] : b[i];
  const uint32_t d0 = (j & 2) ? c[2] : c[0], d1 = (j & 2) ? c[3] : c[1];
  return (j & 1) ? d1 : d0;
}

// The columns of a 32-column slice that cleared the threshold (`hits`):
// v holds raw accumulators (RAW, BF16 forms) or finished distances.  Dense
// mode stores every column at its row's slot; filter mode stages the hits that
// pass the exact key test in this thread's shared-memory column.
template <int MT, int MODE, bool RAW>
__device__ __forceinline__ float drain_dist(uint32_t bits, float qa) {
  const float a = __uint_as_float(bits);
  return !RAW ? a : MT == M_L2 ? fmaf(-2.0f, a, qa) : (MT == M_IP ? a : -a);
}

// One 32-byte store (four keys) to a 32-byte aligned address.
__device__ __forceinline__ void st_global_32b(uint64_t *dst, const uint64_t (&k)[4]) {
  asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(dst), "l"(k[0]), "l"(k[1]), "l"(k[2]),
               "l"(k[3])
               : "memory");
}

// Appends the staged keys to the query's list: one atomic reserves the slots.
__device__ __forceinline__ void flush_hits(const DrainCtx &c, int &nb) {
  uint32_t slot = atomicAdd(c.count + c.qid, (uint32_t)nb);
  uint64_t *out = c.cand + c.qid * c.cap;
  for (int i = 0; i < nb; ++i, ++slot)
    if (slot < (uint32_t)c.cap) out[slot] = c.hb[i * kLpEpiThreads];
  nb = 0;
}

template <int MT, int MODE, bool RAW>
__device__ __forceinline__ void drain_mask(const uint32_t (&v)[32], uint32_t hits, const DrainCtx &c,
                                           int &nb) {
  if constexpr (MODE == TILE_DENSE) {
    uint64_t *out = c.cand + c.qid * c.cap + (c.rt - c.r_begin);
    if (c.rt + 32 <= c.r_end) {
      // a whole slice: 32-byte stores, one full sector each (cap is a
      // multiple of 128 and a slice starts a multiple of 32 rows into the
      // chunk, so `out` is 32-byte aligned)
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        uint64_t kv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) kv[u] = make_key(drain_dist<MT, MODE, RAW>(v[j + u], c.qa), (uint32_t)(c.rt + j + u));
        st_global_32b(out + j, kv);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (c.rt + j < c.r_end) out[j] = make_key(drain_dist<MT, MODE, RAW>(v[j], c.qa), (uint32_t)(c.rt + j));
    }
  } else {
    // the exact key test: only keys below the R-th key are offered, so a
    // rescan after an overflow makes progress even through long runs of ties
    while (hits) {
      const int j = __ffs(hits) - 1;
      hits &= hits - 1;
      const int64_t row = c.rt + j;
      if (row >= c.r_end) continue;
      const float d = drain_dist<MT, MODE, RAW>(pick32(v, j), c.qa);
      if (!(d < c.tau_d || (d == c.tau_d && (uint32_t)row < c.tau_r))) continue;
      c.hb[nb * kLpEpiThreads] = make_key(d, (uint32_t)row);
      if (++nb == kLpHitBuf) flush_hits(c, nb);
    }
  }
}

// A slice's hits in the BF16 filter drain, called by the whole warp
// (converged).  Lanes whose staging column cannot take this slice's hits
// flush it first, all together: one atomic round trip for the warp instead of
// one per lane at different points of a divergent loop.  A lane with more
// hits than the column holds reserves slots for the keys that pass the exact
// key test and stores them directly (only accepted keys are counted, so an
// overflow rescan still makes progress through runs of ties).  The staged loop itself
// never flushes; a full column waits for the next slice or the end of the CTA.
template <int MT>
__device__ __forceinline__ void stage_hits(const uint32_t (&v)[32], uint32_t hits, const DrainCtx &c,
                                           int &nb) {
  const int nh = __popc(hits);
  const bool big = nh > kLpHitBuf;
  const bool must = !big && nb + nh > kLpHitBuf;
  if (__any_sync(0xffffffffu, must)) {
    if (must) flush_hits(c, nb);
  }
  if (__any_sync(0xffffffffu, big)) {
    if (big) {
      uint32_t acc = 0;
      for (uint32_t h = hits; h;) {
        const int j = __ffs(h) - 1;
        h &= h - 1;
        const int64_t row = c.rt + j;
        const float d = drain_dist<MT, TILE_FILTER, true>(pick32(v, j), c.qa);
        if (row < c.r_end && (d < c.tau_d || (d == c.tau_d && (uint32_t)row < c.tau_r))) acc |= 1u << j;
      }
      const int na = __popc(acc);
      uint32_t slot = na ? atomicAdd(c.count + c.qid, (uint32_t)na) : 0u;
      uint64_t *out = c.cand + c.qid * c.cap;
      while (acc) {
        const int j = __ffs(acc) - 1;
        acc &= acc - 1;
        const float d = drain_dist<MT, TILE_FILTER, true>(pick32(v, j), c.qa);
        if (slot < (uint32_t)c.cap) out[slot] = make_key(d, (uint32_t)(c.rt + j));
        ++slot;
      }
    }
  }
  if (big) return;
  while (hits) {
    const int j = __ffs(hits) - 1;
    hits &= hits - 1;
    const int64_t row = c.rt + j;
    if (row >= c.r_end) continue;
    const float d = drain_dist<MT, TILE_FILTER, true>(pick32(v, j), c.qa);
    if (!(d < c.tau_d || (d == c.tau_d && (uint32_t)row < c.tau_r))) continue;
    c.hb[nb * kLpEpiThreads] = make_key(d, (uint32_t)row);
    ++nb;
  }
}

template <int PREC, int MT, int MODE>
__global__ void __launch_bounds__(kLpThreads, 1)
    lowp_tile_kernel(const __grid_constant__ CUtensorMap tmap_a, LpParams p) {
  constexpr bool FOLD = PREC == HORA_PREC_BF16 && MT == M_L2;
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  const int nkb = p.nkb, S = p.stages;
  const uint32_t a_kb_bytes = kLpBM * 128, b_kb_bytes = kLpBN * 128;
  const uint32_t stage_bytes = nkb * b_kb_bytes + (FOLD ? kNormBytesB : 0);
  uint8_t *sA = sm;
  uint8_t *sAn = sm + nkb * a_kb_bytes;  // FOLD: the (1,1,1,0...) block
  uint8_t *sB = sAn + (FOLD ? 4096 : 0);
  uint64_t *bars = reinterpret_cast<uint64_t *>(sB + S * stage_bytes);
  // each ring stage in two halves with their own barriers: K block 0, then
  // the other K blocks and the norm block (when there are any), so the MMA
  // starts on a tile's first half while its second half is still arriving,
  // and a half is refilled as soon as its own MMAs are done
  uint64_t *full = bars, *empty = bars + kLpMaxStages;
  uint64_t *full2 = bars + 2 * kLpMaxStages, *empty2 = bars + 3 * kLpMaxStages;
  uint64_t *a_full = bars + 4 * kLpMaxStages;
  uint64_t *acc_full = a_full + 1, *acc_empty = acc_full + kLpNB, *done = acc_empty + kLpNB;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(done + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q0 = (int64_t)blockIdx.x * kLpBM;
  const int64_t row0 = p.r_begin + (int64_t)blockIdx.y * kLpBN * p.tpc;
  const int64_t rows_here = p.r_end - row0;
  const int T = (int)std::min<int64_t>(p.tpc, (rows_here + kLpBN - 1) / kLpBN);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(full + s, 1);
      tc::mbar_init(empty + s, 1);
      tc::mbar_init(full2 + s, 1);
      tc::mbar_init(empty2 + s, 1);
    }
    tc::mbar_init(a_full, 1);
    for (int b = 0; b < kLpNB; ++b) {
      tc::mbar_init(acc_full + b, 1);
      tc::mbar_init(acc_empty + b, kLpEpiThreads);
    }
    tc::mbar_init(done, 1);
    *abort = 0;
    tc::fence_barrier_init();
  }
  if (FOLD) {
    // A-side norm block: row r = (1, 1, 1, 0, 0, 0, 0, 0 | 0 ... 0)
    uint32_t *w = reinterpret_cast<uint32_t *>(sAn);
    for (int i = threadIdx.x; i < (int)(kNormBytesA / 4); i += blockDim.x) {
      const int word = i & 3;  // 4 words per 16-byte row of the first half
      const bool first_half = i < (int)(kNormHalfA / 4);
      w[i] = !first_half ? 0u : word == 0 ? 0x3F803F80u : word == 1 ? 0x00003F80u : 0u;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, kLpNB * kLpBN);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (tc::elect_one()) {
      tc::prefetch_tmap(&tmap_a);
      const int kb_elems = PREC == HORA_PREC_BF16 ? 64 : 128;
      tc::mbar_arrive_expect_tx(a_full, nkb * a_kb_bytes);
      for (int kb = 0; kb < nkb; ++kb) tc::tma_load_2d(sA + kb * a_kb_bytes, &tmap_a, a_full, kb * kb_elems, (int)q0);
      // base tiles: bulk copies from the tile image, whose bytes are the
      // stage's layout; the first half (K block 0) and the rest separately
      const uint8_t *img = p.tiles + (row0 / kLpBN) * (int64_t)stage_bytes;
      const uint32_t rest = stage_bytes - b_kb_bytes;
      for (int t = 0; t < T; ++t) {
        const int s = t % S, j = t / S;
        uint8_t *st = sB + (size_t)s * stage_bytes;
        const uint8_t *src = img + (int64_t)t * stage_bytes;
        if (j > 0 && !tc::mbar_wait(empty + s, (j - 1) & 1, abort)) break;
        tc::mbar_arrive_expect_tx(full + s, b_kb_bytes);
        tc::bulk_load(st, src, b_kb_bytes, full + s);
        if (rest) {
          if (j > 0 && !tc::mbar_wait(empty2 + s, (j - 1) & 1, abort)) break;
          tc::mbar_arrive_expect_tx(full2 + s, rest);
          tc::bulk_load(st + b_kb_bytes, src + b_kb_bytes, rest, full2 + s);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (tc::elect_one()) {
      constexpr uint32_t idesc = tc::idesc_f32acc(PREC == HORA_PREC_BF16 ? 1u : 0u, kLpBM, kLpBN);
      bool ok = tc::mbar_wait(a_full, 0, abort);
      const bool rest = nkb > 1 || FOLD;  // a second half exists
      for (int t = 0; ok && t < T; ++t) {
        const int s = t % S, j = t / S, b = t % kLpNB, jb = t / kLpNB;
        if (!tc::mbar_wait(full + s, j & 1, abort)) break;
        if (jb > 0 && !tc::mbar_wait(acc_empty + b, (jb - 1) & 1, abort)) break;
        tc::fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(b * kLpBN);
        uint8_t *st = sB + (size_t)s * stage_bytes;
        bool ok2 = true;
        for (int kb = 0; kb < nkb; ++kb) {
          if (kb == 1) {
            // K block 0 read: its half of the stage may be refilled
            tc::mma_commit(empty + s);
            if (!tc::mbar_wait(full2 + s, j & 1, abort)) {
              ok2 = false;
              break;
            }
            tc::fence_after_sync();
          }
          const uint32_t a0 = tc::smem_u32(sA + kb * a_kb_bytes);
          const uint32_t b0 = tc::smem_u32(st + kb * b_kb_bytes);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = tc::sdesc_kmajor_sw128(a0 + kk * 32);
            const uint64_t bd = tc::sdesc_kmajor_sw128(b0 + kk * 32);
            const uint32_t acc = (kb | kk) ? 1u : 0u;
            if (PREC == HORA_PREC_BF16)
              tc::mma_bf16(d, ad, bd, idesc, acc);
            else
              tc::mma_e4m3(d, ad, bd, idesc, acc);
          }
        }
        if (!ok2) break;
        if (FOLD) {
          if (nkb == 1) {
            tc::mma_commit(empty + s);
            if (!tc::mbar_wait(full2 + s, j & 1, abort)) break;
            tc::fence_after_sync();
          }
          const uint64_t ad = tc::sdesc_kmajor_none(tc::smem_u32(sAn), kNormHalfA, 128);
          const uint64_t bd = tc::sdesc_kmajor_none(tc::smem_u32(st + nkb * b_kb_bytes), kNormHalfB, 128);
          tc::mma_bf16(d, ad, bd, idesc, 1u);
        }
        tc::mma_commit(rest ? empty2 + s : empty + s);
        tc::mma_commit(acc_full + b);
      }
      // all MMAs of this thread complete before TMEM is released
      tc::mma_commit(done);
      tc::mbar_wait(done, 0, abort, tc::kWaitCycles, /*ignore_abort=*/true);
    }
  } else {
    // ---------------- drain ----------------
    const int g = warp & 3;           // TMEM lane group this warp may access
    const int h = (warp - 2) >> 2;    // column quarter (32 columns)
    const int m = g * 32 + lane;      // query row in the tile
    const int64_t qrow = q0 + m;
    const int64_t qid = qrow < p.nq ? (p.qmap ? p.qmap[qrow] : qrow) : -1;
    float qa = 0.0f, qs = 1.0f;
    if (qid >= 0) {
      if (MT == M_L2) qa = p.qsq[qid];
      if (MT == M_COS) qa = p.qnorm[qid];
      if (PREC == HORA_PREC_FP8) qs = p.qscale[qid];
    }
    float tau_d = __int_as_float(0x7f800000);
    uint32_t tau_r = 0xffffffffu;  // fewer than R keys yet: every finite distance passes
    if (MODE == TILE_FILTER && qid >= 0) {
      const uint64_t tk = p.best[qid * p.k + (p.k - 1)];
      if (tk != kEmptyKey) {
        tau_d = key_dist(tk);
        tau_r = key_row(tk);
      }
      if (p.tau0) {
        // a probed threshold: every row at or below it is kept
        const float t0 = p.tau0[qid];
        if (t0 < tau_d) {
          tau_d = t0;
          tau_r = 0xffffffffu;
        }
      }
    }
    // BF16: the accumulator is the distance up to a per-query affine map
    // (Euclidean: qsq - 2 acc with the norm folded in; DotProduct: acc;
    // CosineSimilarity on unit rows: -acc), so a column can only be a
    // candidate if acc clears thr; thr is loosened by a relative 1e-6 so no
    // candidate is lost to rounding, and the exact key test runs in the drain.
    constexpr bool FAST = PREC == HORA_PREC_BF16;
    float thr = 0.0f;
    if (FAST && MODE == TILE_FILTER) {
      const float slack = 1e-6f * (fabsf(qa) + fabsf(tau_d)) + 1e-30f;
      thr = MT == M_L2 ? 0.5f * (qa - tau_d) - slack : (MT == M_IP ? tau_d + slack : -tau_d - slack);
    }
    uint64_t *hbuf = reinterpret_cast<uint64_t *>(bars + kLpBarSlots);
    uint64_t amin = kEmptyKey;  // TILE_ARGMIN: this thread's smallest key so far
    DrainCtx c{p.cand, p.count, hbuf + (threadIdx.x - 64), qid, 0, p.r_begin, p.r_end, p.cap, qa, tau_d, tau_r};
    int nb = 0;  // keys staged in this thread's column
    for (int t = 0; t < T; ++t) {
      const int b = t % kLpNB, jb = t / kLpNB;
      const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(acc_full + b, jb & 1, abort));
      if (!ok) break;
      tc::fence_after_sync();
      // this warp's 32-column slices of the tile, one at a time; the buffer
      // goes back to the MMA as soon as the last slice is in registers
#pragma unroll 1
      for (int sl = 0; sl < kLpSlices; ++sl) {
      // tcgen05.ld is warp-collective: lanes that skipped the previous
      // slice's hit handling wait here for the others
      __syncwarp();
      c.rt = row0 + (int64_t)t * kLpBN + (h * kLpSlices + sl) * 32;
      // generic forms: this lane's row factor, broadcast by shuffle below
      float xa = 0.0f, xs = 1.0f;
      if (!FAST) {
        const int64_t r = c.rt + lane;
        const float *va = MT == M_L2 ? p.xsq : (MT == M_COS ? p.xnorm : nullptr);
        if (va) xa = r < p.r_end ? __ldg(va + r) : 0.0f;
        if (PREC == HORA_PREC_FP8) xs = r < p.r_end ? __ldg(p.xscale + r) : 0.0f;
      }
      uint32_t v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(b * kLpBN + (h * kLpSlices + sl) * 32), v);
      tc::tmem_ld_wait();
      if (sl == kLpSlices - 1) {
        tc::fence_before_sync();
        tc::mbar_arrive(acc_empty + b);
      }
      if (FAST) {
        if constexpr (MODE == TILE_ARGMIN) {
          // the smallest (distance, row) key of the slice: strict < keeps the
          // lowest column among equal distances
          if (qid >= 0) {
            float dm = __int_as_float(0x7f800000);
            int jm = -1;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float d = drain_dist<MT, TILE_DENSE, true>(v[j], qa);
              if (c.rt + j < c.r_end && d < dm) {
                dm = d;
                jm = j;
              }
            }
            if (jm >= 0) {
              const uint64_t key = make_key(dm, (uint32_t)(c.rt + jm));
              amin = key < amin ? key : amin;
            }
          }
        } else if constexpr (MODE == TILE_DENSE) {
          if (qid >= 0) drain_mask<MT, MODE, true>(v, 0xffffffffu, c, nb);
        } else {
          // the slice's extreme decides whether any column can hit; the
          // hit mask is built only then (padded query rows never hit)
          const float ext = slice_extreme<MT == M_IP>(v);
          const bool maybe = qid >= 0 && (MT == M_IP ? ext <= thr : ext >= thr);
          if (p.dense_hits) {
            // many hits per slice: flushes converged across the warp
            if (__any_sync(0xffffffffu, maybe)) {
              uint32_t hits = 0;
              if (maybe) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                  const float a = __uint_as_float(v[j]);
                  hits |= (uint32_t)(MT == M_IP ? a <= thr : a >= thr) << j;
                }
              }
              stage_hits<MT>(v, hits, c, nb);
            }
          } else if (maybe) {
            uint32_t hits = 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float a = __uint_as_float(v[j]);
              hits |= (uint32_t)(MT == M_IP ? a <= thr : a >= thr) << j;
            }
            drain_mask<MT, MODE, true>(v, hits, c, nb);
          }
        }
        continue;
      }
      // finished distances replace the accumulators in place
      uint32_t hits = 0;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        float dot = __uint_as_float(v[j]);
        if (PREC == HORA_PREC_FP8) dot *= qs * __shfl_sync(0xffffffffu, xs, j);
        float d;
        if (MT == M_L2) {
          d = fmaf(-2.0f, dot, qa + __shfl_sync(0xffffffffu, xa, j));
        } else if (MT == M_IP) {
          d = dot;
        } else {
          float den = qa * __shfl_sync(0xffffffffu, xa, j);
          d = den == 0.0f ? 0.0f : -dot / den;
        }
        v[j] = __float_as_uint(d);
        hits |= (uint32_t)(d <= tau_d) << j;
      }
      if (MODE == TILE_DENSE) hits = 0xffffffffu;
      if (qid >= 0 && hits) drain_mask<MT, MODE, false>(v, hits, c, nb);
      }
    }
    if (qid >= 0 && nb > 0) flush_hits(c, nb);
    if (MODE == TILE_ARGMIN && qid >= 0 && amin != kEmptyKey)
      atomicMin(reinterpret_cast<unsigned long long *>(p.best + qid), (unsigned long long)amin);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kLpNB * kLpBN);
  }
  if (threadIdx.x == 0 && *abort) atomicExch(p.err, 1);
}

// ---- conversions -------------------------------------------------------------------
// sq != nullptr scales row r by 1/sqrt(sq[r]) (unit rows; zero rows stay 0)
__global__ void to_bf16_kernel(const float *X, int64_t n, int64_t ld, int64_t dim, int64_t Dp,
                               const double *sq, __nv_bfloat16 *out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * Dp) return;
  int64_t r = i / Dp, t = i % Dp;
  float v = t < dim ? X[r * ld + t] : 0.0f;
  if (sq) v = sq[r] > 0.0 ? (float)((double)v / sqrt(sq[r])) : 0.0f;
  out[i] = __float2bfloat16_rn(v);
}

// -|x|^2 / 2 as h1 + h2 + h3 in BF16 (24 bits, the f32 value), columns 3..15 zero
__global__ void norm_block_kernel(const double *sq, int64_t n, __nv_bfloat16 *out) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float v = (float)(-0.5 * sq[r]);
  __nv_bfloat16 h1 = __float2bfloat16_rn(v);
  float r1 = v - __bfloat162float(h1);
  __nv_bfloat16 h2 = __float2bfloat16_rn(r1);
  float r2 = r1 - __bfloat162float(h2);
  __nv_bfloat16 h3 = __float2bfloat16_rn(r2);
  __nv_bfloat16 *o = out + r * 16;
  o[0] = h1;
  o[1] = h2;
  o[2] = h3;
  for (int i = 3; i < 16; ++i) o[i] = __float2bfloat16_rn(0.0f);
}

// The largest Euclidean norm of x - bf16(x) over the rows (one warp per row,
// f64 sums, rounded up to the next f32) into *out as ordered bits.
__global__ void bf16_residual_max_kernel(const float *X, int64_t n, int64_t ld, int64_t dim, unsigned *out) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  double acc = 0.0;
  for (int64_t t = lane; t < dim; t += 32) {
    const float x = X[r * ld + t];
    const double e = (double)x - (double)__bfloat162float(__float2bfloat16_rn(x));
    acc += e * e;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) atomicMax(out, __float_as_uint(nextafterf((float)sqrt(acc), INFINITY)));
}

// one warp per row: per-row absmax scale so the row's largest entry maps to 448
__global__ void to_e4m3_kernel(const float *X, int64_t n, int64_t ld, int64_t dim, int64_t Dp,
                               uint8_t *out, float *scale) {
  int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (r >= n) return;
  float mx = 0.0f;
  for (int64_t t = lane; t < dim; t += 32) mx = fmaxf(mx, fabsf(X[r * ld + t]));
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  float s = mx > 0.0f ? mx / 448.0f : 1.0f;
  float inv = 1.0f / s;
  for (int64_t t = lane; t < Dp; t += 32) {
    float v = t < dim ? X[r * ld + t] * inv : 0.0f;
    out[r * Dp + t] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
  }
  if (lane == 0) scale[r] = s;
}

__global__ void f64_to_f32_kernel(const double *a, int64_t n, float *out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)a[i];
}

__global__ void gather_rows_u8_kernel(const uint8_t *src, int64_t row_bytes, const int *rows,
                                      int64_t n, uint8_t *dst) {
  int64_t r = blockIdx.x;
  if (r >= n) return;
  const uint8_t *s = src + (int64_t)rows[r] * row_bytes;
  for (int64_t t = threadIdx.x; t < row_bytes; t += blockDim.x) dst[r * row_bytes + t] = s[t];
}

// ---- starting thresholds from pivot clusters (BF16 Euclidean) ---------------------------
// With a threshold that starts at the R-th key of the rows scanned so far,
// the chunked schedule keeps about R x ln(n / first chunk) rows per query
// (~1,500 on 1M rows, R = 132), and the drain's hit handling is the largest
// cost of the scan after the MMAs.  A base of at least kProbeMinRows rows
// therefore keeps ~n / 1,024 pivot clusters (a few Lloyd steps from evenly
// spaced rows).  Before the scan every query goes to its nearest pivot and
// is scored against up to kProbeMaxMembers rows of that cluster with the
// scan's own arithmetic (BF16 operands, exact products, f32 sums, the
// folded norm).  Its starting threshold is the R-th of those distances plus
// a bound on what the different summation order can change; one filter pass
// over the base then keeps every row at or below it.  A query that kept at
// least R rows has its R-best set complete: R rows at or below the
// threshold put its R-th key there, and every key up to that one was kept.
// A query that kept fewer (the bound did not hold, or its cluster had fewer
// than R members) is answered again by the chunked schedule.
constexpr int64_t kProbeRowsPerPivot = 1024;
constexpr int64_t kProbeMinRows = 65536;
constexpr int kProbeMaxMembers = 1024;  // members a query is scored against
constexpr int kProbeMaxR = 256;         // widest R-best list the probe serves
constexpr int kExactTcMaxK = 256;       // largest k of the certified exact search
constexpr int kProbeMinCluster = 256;   // smaller clusters are dissolved at the end
constexpr int kProbeReseed = 128;       // Lloyd steps re-seed clusters below this
constexpr int kProbeLloyd = 6;
constexpr int kProbeQ = 32;       // queries per pass of a probe CTA
constexpr int kProbeRows = 128;   // member rows per shared-memory tile
constexpr int kProbePitch = 132;  // f32 pitch of a staged row (spreads the banks)
constexpr int kProbeSmem = (kProbeQ + kProbeRows) * kProbePitch * 4 + kProbeMaxMembers * 12;

__device__ __forceinline__ void bf16x8_to_f32(const uint4 &v, float *out) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    out[2 * i] = __uint_as_float(w[i] << 16);
    out[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

// The 16 e4m3 values of a 16-byte chunk as f32 (through the library's
// FP8 -> half conversion, exact).
__device__ __forceinline__ void e4m3x16_to_f32(const uint4 &v, float *out) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const __nv_fp8_storage_t b = (__nv_fp8_storage_t)((w[i >> 2] >> (8 * (i & 3))) & 0xffu);
    out[i] = __half2float(__half(__nv_cvt_fp8_to_halfraw(b, __NV_E4M3)));
  }
}

// Elements per 16-byte chunk of a row: 8 BF16 values or 16 e4m3 values.
template <bool FP8>
__device__ __forceinline__ void chunk_to_f32(const uint4 &v, float *out) {
  if (FP8) e4m3x16_to_f32(v, out); else bf16x8_to_f32(v, out);
}

// The 16-byte chunks of member rows mt.. (kProbeRows of them) that thread t
// stages: chunk i = t + 256 u is row i / nch, chunk i % nch.
__device__ __forceinline__ void probe_load_tile(uint4 (&buf)[8], const uint32_t *ids, int mt, int L, int nch, int t,
                                                const uint8_t *tiles, int64_t tile_bytes) {
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int i = t + 256 * u, j = i / nch, ch = i % nch;
    buf[u] = make_uint4(0u, 0u, 0u, 0u);
    if (i < kProbeRows * nch && mt + j < L) {
      const uint32_t r = ids[mt + j];
      const int rr = (int)(r % kLpBN), kb = ch >> 3, cc = ch & 7;
      buf[u] = *reinterpret_cast<const uint4 *>(tiles + (int64_t)(r / kLpBN) * tile_bytes + kb * (kLpBN * 128) +
                                                rr * 128 + ((cc ^ (rr & 7)) * 16));
    }
  }
}

// One CTA per work item: up to kProbeQ of one pivot's queries against its
// first kProbeMaxMembers member rows, read from the tile image.  Thread (qg, rg)
// of the 8 x 32 layout scores queries qg + 8i against rows rg + 32j, the
// products summed over ascending dimensions with one f32 FMA each, then the
// scan's distance formed from the sum: BF16 (norm folded) qsq - 2 (sum +
// (-|x|^2 / 2)); FP8 (per-row scales) qsq + |x|^2 - 2 sum (qscale xscale).
template <bool FP8>
__global__ void __launch_bounds__(256) probe_dist_kernel(const uint8_t *tiles, int64_t tile_bytes,
                                                         const float *xsq, const float *xscale,
                                                         const int64_t *coff, const uint32_t *cmem,
                                                         const uint8_t *lq, const float *lqscale,
                                                         int64_t Dp, const float *qsq, const int64_t *qoff,
                                                         const uint32_t *qmem, const int *item_off, int C,
                                                         float *pdist) {
  extern __shared__ __align__(16) float psm[];
  float *qs = psm;                           // kProbeQ x kProbePitch
  float *xs = qs + kProbeQ * kProbePitch;    // kProbeRows x kProbePitch
  float *xh = xs + kProbeRows * kProbePitch;                       // per member: -|x|^2 / 2 (FP8: |x|^2)
  float *xc = xh + kProbeMaxMembers;                               // per member: its scale (FP8)
  uint32_t *ids = reinterpret_cast<uint32_t *>(xc + kProbeMaxMembers);  // per member: its row
  constexpr int kPer = FP8 ? 16 : 8;  // elements per 16-byte chunk
  constexpr int esz = FP8 ? 1 : 2;
  // work item blockIdx.x: batch (item - item_off[c]) of pivot c's queries
  const int b = blockIdx.x;
  if (b >= item_off[C]) return;
  int lo = 0, hi = C;  // the last c with item_off[c] <= b
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (item_off[mid] <= b) lo = mid; else hi = mid;
  }
  const int c = lo;
  const int64_t q_lo = qoff[c], nqc = qoff[c + 1] - q_lo;
  const int64_t m_lo = coff[c];
  const int L = (int)(coff[c + 1] - m_lo < kProbeMaxMembers ? coff[c + 1] - m_lo : kProbeMaxMembers);
  const int t = threadIdx.x, qg = t & 7, rg = t >> 3;
  const int D = (int)Dp, nch = D / kPer;
  {
    const int64_t qb = (int64_t)(b - item_off[c]) * kProbeQ;
    const int nb = (int)(nqc - qb < kProbeQ ? nqc - qb : kProbeQ);
    const int ni = (nb + 7) >> 3;  // query slots in use per thread (CTA-uniform)
    for (int j = t; j < L; j += 256) {
      const uint32_t r = cmem[m_lo + j];
      ids[j] = r;
      xh[j] = FP8 ? xsq[r] : -0.5f * xsq[r];
      xc[j] = FP8 ? xscale[r] : 1.0f;
    }
    for (int i = t; i < kProbeQ * nch; i += 256) {
      const int qi = i / nch, ch = i % nch;
      float f[16];
#pragma unroll
      for (int e = 0; e < kPer; ++e) f[e] = 0.0f;
      if (qi < nb) {
        const uint32_t qid = qmem[q_lo + qb + qi];
        chunk_to_f32<FP8>(*reinterpret_cast<const uint4 *>(lq + ((int64_t)qid * Dp + ch * kPer) * esz), f);
      }
      float4 *dst = reinterpret_cast<float4 *>(qs + qi * kProbePitch + ch * kPer);
#pragma unroll
      for (int e = 0; e < kPer / 4; ++e) dst[e] = make_float4(f[4 * e], f[4 * e + 1], f[4 * e + 2], f[4 * e + 3]);
    }
    __syncthreads();  // member rows and queries staged
    // a tile's 16-byte chunks in registers: the next tile's loads are in
    // flight while the current one is scored
    uint4 buf[8];
    probe_load_tile(buf, ids, 0, L, nch, t, tiles, tile_bytes);
    for (int mt = 0; mt < L; mt += kProbeRows) {
      if (mt > 0) __syncthreads();  // the previous tile consumed
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int i = t + 256 * u, j = i / nch, ch = i % nch;
        if (i < kProbeRows * nch) {
          float f[16];
          chunk_to_f32<FP8>(buf[u], f);
          float4 *dst = reinterpret_cast<float4 *>(xs + j * kProbePitch + ch * kPer);
#pragma unroll
          for (int e = 0; e < kPer / 4; ++e) dst[e] = make_float4(f[4 * e], f[4 * e + 1], f[4 * e + 2], f[4 * e + 3]);
        }
      }
      __syncthreads();
      if (mt + kProbeRows < L) probe_load_tile(buf, ids, mt + kProbeRows, L, nch, t, tiles, tile_bytes);
      float acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
#pragma unroll 2
      for (int d = 0; d < D; d += 4) {
        float4 xv[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) xv[j] = *reinterpret_cast<const float4 *>(xs + (rg + 32 * j) * kProbePitch + d);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          if (i < ni) {
            const float4 qv = *reinterpret_cast<const float4 *>(qs + (qg + 8 * i) * kProbePitch + d);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              acc[i][j] = fmaf(qv.x, xv[j].x, acc[i][j]);
              acc[i][j] = fmaf(qv.y, xv[j].y, acc[i][j]);
              acc[i][j] = fmaf(qv.z, xv[j].z, acc[i][j]);
              acc[i][j] = fmaf(qv.w, xv[j].w, acc[i][j]);
            }
          }
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int qi = qg + 8 * i;
        if (i >= ni || qi >= nb) continue;
        const uint32_t qid = qmem[q_lo + qb + qi];
        const float qa = qsq[qid];
        const float qsc = FP8 ? lqscale[qid] : 1.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int m = mt + rg + 32 * j;
          if (m < L)
            pdist[(int64_t)qid * kProbeMaxMembers + m] =
                FP8 ? fmaf(-2.0f, acc[i][j] * (qsc * xc[m]), qa + xh[m]) : fmaf(-2.0f, acc[i][j] + xh[m], qa);
        }
      }
    }
  }
}

// One warp per query: the R-th smallest probe distance by a 32-step bitwise
// descent over the ordered encoding, plus the summation-order bound
// 1e-4 (|q|^2 + max |x|^2).  Both sums add the same exact BF16 products
// (<= |q||x| + |x|^2 / 2 in magnitude, <= |q|^2 / 2 + max|x|^2) in f32; each
// is within 144 x 2^-24 of that magnitude, so the distances (2 x the sum)
// differ by less than 3.5e-5 of it.  A cluster with fewer than R members
// gives -FLT_MAX: the scan keeps nothing and the query is rescheduled.
__global__ void probe_select_kernel(const uint64_t *pkeys, const int64_t *coff, const float *pdist,
                                    const float *qsq, const float *xsqmax, int64_t nq, int R,
                                    const float *slack, float *tau) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const uint32_t c = key_row(pkeys[q]);
  const int L = (int)(coff[c + 1] - coff[c] < kProbeMaxMembers ? coff[c + 1] - coff[c] : kProbeMaxMembers);
  if (L < R) {
    if (lane == 0) tau[q] = -FLT_MAX;
    return;
  }
  uint32_t v[kProbeMaxMembers / 32];
#pragma unroll
  for (int i = 0; i < kProbeMaxMembers / 32; ++i) {
    const int m = lane + 32 * i;
    v[i] = m < L ? f2ord(pdist[q * kProbeMaxMembers + m]) : 0xffffffffu;
  }
  // the largest a with fewer than R values below it is the R-th smallest;
  // the descent stops kSelectSkip bits short and rounds up (an upper bound
  // within 2^-(23 - kSelectSkip) of the value, which is all a threshold needs)
  constexpr int kSelectSkip = 12;
  uint32_t a = 0;
  for (int b = 31; b >= kSelectSkip; --b) {
    const uint32_t tt = a | (1u << b);
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < kProbeMaxMembers / 32; ++i) cnt += v[i] < tt;
#pragma unroll
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (cnt < R) a = tt;
  }
  if (lane == 0) {
    float t = ord2f(a | ((1u << kSelectSkip) - 1)) + 1e-4f * (qsq[q] + *xsqmax);
    // the certified exact search widens it by its error bound (and by a
    // relative 2^-20 against the rounding of these f32 additions)
    if (slack) t = t + slack[q] + 0x1p-20f * fabsf(t + slack[q]);
    tau[q] = t;
  }
}

// Probe work items: pivot c owns ceil(queries / kProbeQ) of them, from
// item_off[c] (C + 1 offsets; one CTA of 1,024 threads, C <= 4,096).
__global__ void probe_items_kernel(const int64_t *qoff, int C, int *item_off) {
  __shared__ int part[1024];
  const int t = threadIdx.x, per = (C + 1023) / 1024;
  const int lo = min(C, t * per), hi = min(C, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += (int)((qoff[c + 1] - qoff[c] + kProbeQ - 1) / kProbeQ);
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int i = 0; i < 1024; ++i) {
      const int v = part[i];
      part[i] = run;
      run += v;
    }
    item_off[C] = run;
  }
  __syncthreads();
  int run = part[t];
  for (int c = lo; c < hi; ++c) {
    item_off[c] = run;
    run += (int)((qoff[c + 1] - qoff[c] + kProbeQ - 1) / kProbeQ);
  }
}

// Re-seeds centre dst[i] with base row cmem[src[i]] (all ld columns).
__global__ void reseed_kernel(const float *X, int64_t ld, const uint32_t *cmem, const int64_t *src,
                              const int *dst, int m, float *centers) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)m * ld) return;
  const int j = (int)(i / ld);
  centers[(int64_t)dst[j] * ld + (i % ld)] = X[(int64_t)cmem[src[j]] * ld + (i % ld)];
}

// Queries whose R-best list is still short after the probed pass, appended
// to list (count in *n).
__global__ void short_lists_kernel(const uint64_t *best, int R, int64_t nq, int *n, int *list) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && best[q * R + (R - 1)] == kEmptyKey) list[atomicAdd(n, 1)] = (int)q;
}

// Empties the R-best lists of the listed queries.
__global__ void clear_lists_kernel(uint64_t *best, int R, const int *list, int64_t nl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl * R) best[(int64_t)list[i / R] * R + (i % R)] = kEmptyKey;
}

// The largest of n non-negative floats (as ordered bits) into *out.
__global__ void max_nonneg_kernel(const float *x, int64_t n, unsigned *out) {
  float m = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, x[i]);
#pragma unroll
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// Pivots of clusters below kProbeMinCluster members are moved out of reach
// so that the final assignment spreads their rows over the others.
__global__ void dissolve_small_kernel(float *centers, int64_t ld, int64_t dim, const int64_t *counts, int C) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)C * dim) return;
  const int c = (int)(i / dim);
  if (counts[c] < kProbeMinCluster) centers[(int64_t)c * ld + (i % dim)] = 1e15f;
}

// ---- host ------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int encode_fn(EncodeTiledFn *out) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
      return fail(HORA_ECUDA, "cuTensorMapEncodeTiled unavailable");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  *out = fn;
  return HORA_OK;
}

// 2-D K-major map: rows x row_bytes, box = 128 bytes x box_rows, 128B swizzle.
static int make_tmap(CUtensorMap *m, const void *ptr, int prec, int64_t Dp, int64_t rows,
                     uint32_t box_rows) {
  EncodeTiledFn enc;
  HORA_TRY(encode_fn(&enc));
  const bool bf = prec == HORA_PREC_BF16;
  const uint64_t esz = bf ? 2 : 1;
  cuuint64_t dims[2] = {(cuuint64_t)Dp, (cuuint64_t)std::max<int64_t>(rows, 1)};
  cuuint64_t strides[1] = {(cuuint64_t)(Dp * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, bf ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                   const_cast<void *>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(HORA_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return HORA_OK;
}

static int lp_smem_bytes(int nkb, int stages, bool fold) {
  return 1024 + nkb * kLpBM * 128 + (fold ? 4096 : 0) +
         stages * (nkb * kLpBN * 128 + (fold ? (int)kNormBytesB : 0)) + kLpBarSlots * 8 + kLpHitBytes;
}

// Ring depth: as many base tiles as fit in ~220 KB of shared memory beside
// the query tile and the hit staging.
static int lp_stages(int nkb, bool fold) {
  const int fixed = 1024 + nkb * kLpBM * 128 + (fold ? 4096 : 0) + kLpBarSlots * 8 + kLpHitBytes;
  const int stage = nkb * kLpBN * 128 + (fold ? (int)kNormBytesB : 0);
  return std::max(2, std::min(kLpMaxStages, (220 * 1024 - fixed) / stage));
}

// The largest tiles-per-CTA of 32 / 16 / 8 whose grid still holds two
// waves of CTAs (one CTA per SM), else 8.
static int lp_tiles_per_cta(int64_t nq, int64_t rows) {
  const int64_t qb = ceil_div(nq, kLpBM);
  for (int tpc = kLpTilesPerCta; tpc > kLpMinTilesPerCta; tpc >>= 1)
    if (qb * ceil_div(rows, (int64_t)kLpBN * tpc) >= 2 * 152) return tpc;
  return kLpMinTilesPerCta;
}

template <int PREC, int MT, int MODE>
static int launch_lp3(const CUtensorMap &ta, const LpParams &p, cudaStream_t s) {
  const int smem = lp_smem_bytes(p.nkb, p.stages, PREC == HORA_PREC_BF16 && MT == M_L2);
  HORA_SMEM_ATTR((lowp_tile_kernel<PREC, MT, MODE>), smem);
  const int64_t rows = p.r_end - p.r_begin;
  dim3 grid((unsigned)ceil_div(p.nq, kLpBM), (unsigned)ceil_div(rows, (int64_t)kLpBN * p.tpc));
  if (grid.x == 0 || grid.y == 0) return HORA_OK;
  ProfScope ps(PREC == HORA_PREC_BF16 ? "bf16_tc_scan" : "fp8_tc_scan", s);
  lowp_tile_kernel<PREC, MT, MODE><<<grid, kLpThreads, smem, s>>>(ta, p);
  HORA_LAUNCHED();
  return HORA_OK;
}

template <int PREC>
static int launch_lp2(int metric, int mode, const CUtensorMap &ta, const LpParams &p, cudaStream_t s) {
  const bool dense = mode == TILE_DENSE;
  switch (metric) {
    case M_L2: return dense ? launch_lp3<PREC, M_L2, TILE_DENSE>(ta, p, s) : launch_lp3<PREC, M_L2, TILE_FILTER>(ta, p, s);
    case M_IP: return dense ? launch_lp3<PREC, M_IP, TILE_DENSE>(ta, p, s) : launch_lp3<PREC, M_IP, TILE_FILTER>(ta, p, s);
    case M_COS: return dense ? launch_lp3<PREC, M_COS, TILE_DENSE>(ta, p, s) : launch_lp3<PREC, M_COS, TILE_FILTER>(ta, p, s);
  }
  return fail(HORA_EMETRIC, "no tensor-core form for this metric");
}

static int launch_lp(int prec, int metric, int mode, const CUtensorMap &ta, const LowpState &L,
                     const LpParams &p, cudaStream_t s) {
  LpParams q = p;
  q.tiles = L.tiles.as<uint8_t>();
  return prec == HORA_PREC_BF16 ? launch_lp2<HORA_PREC_BF16>(metric, mode, ta, q, s)
                                : launch_lp2<HORA_PREC_FP8>(metric, mode, ta, q, s);
}

// The tile image from a row-major copy (n x row_bytes) and, for BF16
// Euclidean, the n x 32-byte norm block: one thread per 16-byte chunk.
__global__ void tile_image_kernel(const uint8_t *rows, int64_t n, int64_t row_bytes, int nkb,
                                  const uint8_t *norm, int64_t tile_bytes, int64_t ntiles, uint8_t *out) {
  const int64_t per_tile = (int64_t)kLpBN * (nkb * 8 + (norm ? 2 : 0));
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntiles * per_tile) return;
  const int64_t t = i / per_tile;
  const int64_t w = i % per_tile;
  uint8_t *tile = out + t * tile_bytes;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (w < (int64_t)kLpBN * nkb * 8) {
    const int kb = (int)(w / (kLpBN * 8));
    const int r = (int)((w / 8) % kLpBN), c = (int)(w % 8);
    const int64_t row = t * kLpBN + r;
    if (row < n) v = *reinterpret_cast<const uint4 *>(rows + row * row_bytes + kb * 128 + c * 16);
    *reinterpret_cast<uint4 *>(tile + kb * (kLpBN * 128) + r * 128 + ((c ^ (r & 7)) * 16)) = v;
  } else {
    const int64_t u = w - (int64_t)kLpBN * nkb * 8;
    const int half = (int)(u / kLpBN), r = (int)(u % kLpBN);
    const int64_t row = t * kLpBN + r;
    if (row < n) v = *reinterpret_cast<const uint4 *>(norm + row * 32 + half * 16);
    *reinterpret_cast<uint4 *>(tile + nkb * (kLpBN * 128) + half * (kLpBN * 16) + r * 16) = v;
  }
}

// Low-precision copy of the base (and its exact squared norms / scales),
// rebuilt when the precision or the item count changes.
static int ensure_lowp(hora_index *h, int prec, cudaStream_t s) {
  const int64_t kbe = prec == HORA_PREC_BF16 ? 64 : 128;
  const int64_t Dp = round_up((int64_t)h->dim, kbe);
  if (h->lowp && h->lowp->prec == prec && h->lowp->n == h->n && h->lowp->metric == h->metric)
    return HORA_OK;
  std::unique_ptr<LowpState, LowpDeleter> st(new LowpState());
  st->prec = prec;
  st->metric = h->metric;
  st->n = h->n;
  st->Dp = Dp;
  const int64_t esz = prec == HORA_PREC_BF16 ? 2 : 1;
  const int nkb = (int)(Dp / kbe);
  const bool fold = prec == HORA_PREC_BF16 && h->metric == M_L2;
  st->tile_bytes = (int64_t)nkb * kLpBN * 128 + (fold ? (int64_t)kNormBytesB : 0);
  const int64_t ntiles = std::max<int64_t>(ceil_div(h->n, kLpBN), 1);
  DevBuf rows, normblk;  // row-major staging, freed once the image is built
  HORA_TRY(rows.reserve(std::max<int64_t>(h->n, 1) * Dp * esz));
  HORA_TRY(st->tiles.reserve(ntiles * st->tile_bytes));
  HORA_TRY(st->xsq.reserve(sizeof(float) * std::max<int64_t>(h->n, 1)));
  {
    ProfScope ps("lowp_convert", s);
    if (prec == HORA_PREC_BF16) {
      to_bf16_kernel<<<ceil_div(h->n * Dp, 256), 256, 0, s>>>(
          h->base.as<float>(), h->n, h->ld, h->dim, Dp,
          h->metric == M_COS ? h->xsq64.as<double>() : nullptr, rows.as<__nv_bfloat16>());
      if (fold) {
        HORA_LAUNCHED();
        HORA_TRY(normblk.reserve(std::max<int64_t>(h->n, 1) * 16 * 2));
        norm_block_kernel<<<ceil_div(h->n, 256), 256, 0, s>>>(h->xsq64.as<double>(), h->n,
                                                              normblk.as<__nv_bfloat16>());
        HORA_LAUNCHED();
        HORA_TRY(st->dxmax.reserve(sizeof(float)));
        HORA_CUDA_TRY(cudaMemsetAsync(st->dxmax.ptr, 0, sizeof(float), s));
        bf16_residual_max_kernel<<<ceil_div(h->n, 8), 256, 0, s>>>(h->base.as<float>(), h->n, h->ld, h->dim,
                                                                   st->dxmax.as<unsigned>());
      }
    } else {
      HORA_TRY(st->xscale.reserve(sizeof(float) * std::max<int64_t>(h->n, 1)));
      to_e4m3_kernel<<<ceil_div(h->n, 8), 256, 0, s>>>(h->base.as<float>(), h->n, h->ld, h->dim, Dp,
                                                       rows.as<uint8_t>(), st->xscale.as<float>());
    }
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<ceil_div(h->n, 256), 256, 0, s>>>(h->xsq64.as<double>(), h->n, st->xsq.as<float>());
    HORA_LAUNCHED();
    const int64_t chunks = ntiles * kLpBN * (nkb * 8 + (fold ? 2 : 0));
    tile_image_kernel<<<ceil_div(chunks, 256), 256, 0, s>>>(rows.as<uint8_t>(), h->n, Dp * esz, nkb,
                                                            fold ? normblk.as<uint8_t>() : nullptr,
                                                            st->tile_bytes, ntiles, st->tiles.as<uint8_t>());
    HORA_LAUNCHED();
  }
  HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the staging buffers are freed on return
  h->lowp = std::move(st);
  return HORA_OK;
}

// Pivots of an n-row base: ~n / kProbeRowsPerPivot, 16 to 4,096.
static int probe_pivot_count(int64_t n) {
  return (int)std::min<int64_t>(4096, std::max<int64_t>(16, n / kProbeRowsPerPivot));
}

static bool probe_eligible(const hora_index *h) {
  return h->bf_probe && (h->precision == HORA_PREC_BF16 || h->precision == HORA_PREC_FP8) && h->metric == M_L2 &&
         h->n >= kProbeMinRows;
}

// Pivot clusters of the base (exact FP32 nearest-pivot assignment): evenly
// spaced rows, then kProbeLloyd Lloyd steps in which a cluster below
// kProbeReseed members is re-seeded with a member of one of the largest
// clusters (so that clusters which absorbed a whole group of rows without a
// pivot of their own get split), then clusters below kProbeMinCluster
// members dissolved into their neighbours by one more assignment.  Built
// once per low-precision state, with the pivots' own BF16 tile image for the
// queries' assignment.
static int ensure_pivots(hora_index *h, LowpState &L, cudaStream_t s) {
  if (L.pc > 0) return HORA_OK;
  const int64_t n = h->n, ld = (int64_t)h->ld;
  const int C = probe_pivot_count(n);
  DevBuf keys, blk, cnt, plan;
  HORA_TRY(L.centers.reserve(sizeof(float) * C * ld));
  HORA_TRY(L.coff.reserve(sizeof(int64_t) * (C + 1)));
  HORA_TRY(L.cmem.reserve(sizeof(uint32_t) * n));
  HORA_TRY(L.xsqmax.reserve(sizeof(float)));
  HORA_TRY(keys.reserve(sizeof(uint64_t) * n));
  HORA_TRY(plan.reserve((sizeof(int64_t) + sizeof(int)) * C));
  std::vector<int64_t> h_cnt(C), h_off(C + 1), h_src;
  std::vector<int> h_dst;
  ProfScope ps("probe_pivots", s);
  const int64_t step = n / C;
  HORA_CUDA_TRY(cudaMemcpy2DAsync(L.centers.ptr, sizeof(float) * ld, h->base.ptr, sizeof(float) * ld * step,
                                  sizeof(float) * ld, C, cudaMemcpyDeviceToDevice, s));
  for (int it = 0; it <= kProbeLloyd + 1; ++it) {
    TileParams p;
    p.Q = h->base.as<float>();
    p.ldq = ld;
    p.nq = n;
    p.X = L.centers.as<float>();
    p.ldx = ld;
    p.r_begin = 0;
    p.r_end = C;
    p.ld = ld;
    p.out_key = keys.as<uint64_t>();
    HORA_TRY(launch_dist_tile(M_L2, TILE_ARGMIN, p, s));
    HORA_TRY(sort_labels(keys.as<uint64_t>(), nullptr, n, C, blk, cnt, L.coff.as<int64_t>(),
                         L.cmem.as<uint32_t>(), s));
    if (it == kProbeLloyd + 1) break;
    if (it == kProbeLloyd) {
      dissolve_small_kernel<<<ceil_div((int64_t)C * h->dim, 256), 256, 0, s>>>(L.centers.as<float>(), ld, h->dim,
                                                                              cnt.as<int64_t>(), C);
      HORA_LAUNCHED();
      continue;
    }
    HORA_TRY(launch_center_sum(h->base.as<float>(), ld, L.cmem.as<uint32_t>(), L.coff.as<int64_t>(), C, h->dim, 0,
                               0.0f, L.centers.as<float>(), s));
    // re-seed the small clusters from the largest ones (host plan)
    HORA_CUDA_TRY(cudaMemcpyAsync(h_cnt.data(), cnt.ptr, sizeof(int64_t) * C, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(h_off.data(), L.coff.ptr, sizeof(int64_t) * (C + 1), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> order(C);
    for (int c = 0; c < C; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return h_cnt[x] > h_cnt[y]; });
    h_src.clear();
    h_dst.clear();
    int big = 0;
    for (int c = 0; c < C; ++c) {
      if (h_cnt[c] >= kProbeReseed) continue;
      const int from = order[big % C];
      if (h_cnt[from] < 4 * kProbeReseed) break;  // nothing large enough to split
      // a member a third of the way into the donor's list (row order)
      h_src.push_back(h_off[from] + h_cnt[from] / 3 + (big / C));
      h_dst.push_back(c);
      ++big;
    }
    if (!h_dst.empty()) {
      const int m = (int)h_dst.size();
      int64_t *d_src = plan.as<int64_t>();
      int *d_dst = reinterpret_cast<int *>(d_src + C);
      HORA_CUDA_TRY(cudaMemcpyAsync(d_src, h_src.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, s));
      HORA_CUDA_TRY(cudaMemcpyAsync(d_dst, h_dst.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s));
      reseed_kernel<<<ceil_div((int64_t)m * ld, 256), 256, 0, s>>>(h->base.as<float>(), ld, L.cmem.as<uint32_t>(),
                                                                  d_src, d_dst, m, L.centers.as<float>());
      HORA_LAUNCHED();
      HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the host plan is reused next step
    }
  }
  HORA_CUDA_TRY(cudaMemsetAsync(L.xsqmax.ptr, 0, sizeof(float), s));
  max_nonneg_kernel<<<152, 256, 0, s>>>(L.xsq.as<float>(), n, L.xsqmax.as<unsigned>());
  HORA_LAUNCHED();
  // the pivots' tile image (BF16 rows and folded norms, like the base's)
  const int64_t Dp = round_up((int64_t)h->dim, 64);  // BF16, whatever the base's precision
  const int nkb = (int)(Dp / 64);
  L.cnkb = nkb;
  L.ctile_bytes = (int64_t)nkb * kLpBN * 128 + kNormBytesB;
  const int64_t ctiles = ceil_div((int64_t)C, (int64_t)kLpBN);
  DevBuf crow, cnorm, csq;
  HORA_TRY(crow.reserve(sizeof(__nv_bfloat16) * C * Dp));
  HORA_TRY(cnorm.reserve(sizeof(__nv_bfloat16) * C * 16));
  HORA_TRY(csq.reserve(sizeof(double) * C));
  HORA_TRY(L.ctiles.reserve(ctiles * L.ctile_bytes));
  HORA_TRY(launch_row_norms(L.centers.as<float>(), C, ld, h->dim, nullptr, csq.as<double>(), s));
  to_bf16_kernel<<<ceil_div((int64_t)C * Dp, 256), 256, 0, s>>>(L.centers.as<float>(), C, ld, h->dim, Dp, nullptr,
                                                                crow.as<__nv_bfloat16>());
  HORA_LAUNCHED();
  norm_block_kernel<<<ceil_div((int64_t)C, 256), 256, 0, s>>>(csq.as<double>(), C, cnorm.as<__nv_bfloat16>());
  HORA_LAUNCHED();
  tile_image_kernel<<<ceil_div(ctiles * kLpBN * (nkb * 8 + 2), 256), 256, 0, s>>>(
      crow.as<uint8_t>(), C, Dp * 2, nkb, cnorm.as<uint8_t>(), L.ctile_bytes, ctiles, L.ctiles.as<uint8_t>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the temporaries are freed on return
  L.pc = C;
  return HORA_OK;
}

// Starting thresholds of nq staged queries (ws.q f32, ws.lq, ws.lqsq) into
// ws.ptau.  lp carries the search's scan parameters; the pivot pass keeps
// each query's nearest pivot key in ws.pkeys.
// ta16: the queries' BF16 tile map (the pivot pass runs in BF16 whatever
// the base's precision); the probe scores members in the base's precision
// (prec), from ws.lq (and ws.lqscale for FP8).
static int probe_thresholds(hora_index *h, LowpState &L, int prec, int64_t nq, int R, int64_t Dp,
                            SearchWorkspace &ws, const CUtensorMap &ta16, const LpParams &lp, cudaStream_t s,
                            const float *slack = nullptr) {
  const int C = L.pc;
  // sized for a power of two of at least 1,024 queries: a serving slot whose
  // batches vary reallocates (and with that waits for the device) rarely
  int64_t nres = 1024;
  while (nres < nq) nres <<= 1;
  HORA_TRY(ws.pkeys.reserve(sizeof(uint64_t) * nres));
  HORA_TRY(ws.poff.reserve(sizeof(int64_t) * (C + 1) + sizeof(int) * (C + 1)));
  HORA_TRY(ws.pmem.reserve(sizeof(uint32_t) * nres));
  HORA_TRY(ws.pdist.reserve(sizeof(float) * nres * kProbeMaxMembers));
  HORA_TRY(ws.ptau.reserve(sizeof(float) * nres));
  int64_t *qoff = ws.poff.as<int64_t>();
  int *item_off = reinterpret_cast<int *>(qoff + C + 1);
  // nearest pivot: the tensor-core scan over the pivots in dense mode, then the best key
  LpParams a = lp;
  a.tiles = L.ctiles.as<uint8_t>();
  a.r_begin = 0;
  a.r_end = C;
  a.tpc = lp_tiles_per_cta(nq, C);
  a.tau0 = nullptr;
  a.dense_hits = 0;
  a.nkb = L.cnkb;
  a.stages = lp_stages(L.cnkb, true);
  // each drain thread's smallest key, combined by a 64-bit atomic minimum
  // per query (no per-pivot keys written)
  a.best = ws.pkeys.as<uint64_t>();
  HORA_CUDA_TRY(cudaMemsetAsync(ws.pkeys.ptr, 0xff, sizeof(uint64_t) * nq, s));
  HORA_TRY((launch_lp3<HORA_PREC_BF16, M_L2, TILE_ARGMIN>(ta16, a, s)));
  HORA_TRY(sort_labels(ws.pkeys.as<uint64_t>(), nullptr, nq, C, ws.pblk, ws.pcnt, qoff, ws.pmem.as<uint32_t>(), s));
  const bool fp8 = prec == HORA_PREC_FP8;
  if (fp8)
    HORA_SMEM_ATTR(probe_dist_kernel<true>, kProbeSmem);
  else
    HORA_SMEM_ATTR(probe_dist_kernel<false>, kProbeSmem);
  {
    ProfScope ps("probe_scores", s);
    probe_items_kernel<<<1, 1024, 0, s>>>(qoff, C, item_off);
    HORA_LAUNCHED();
    const unsigned grid = (unsigned)(C + ceil_div(nq, (int64_t)kProbeQ));
    if (fp8)
      probe_dist_kernel<true><<<grid, 256, kProbeSmem, s>>>(
          L.tiles.as<uint8_t>(), L.tile_bytes, L.xsq.as<float>(), L.xscale.as<float>(), L.coff.as<int64_t>(),
          L.cmem.as<uint32_t>(), ws.lq.as<uint8_t>(), ws.lqscale.as<float>(), Dp, ws.lqsq.as<float>(), qoff,
          ws.pmem.as<uint32_t>(), item_off, C, ws.pdist.as<float>());
    else
      probe_dist_kernel<false><<<grid, 256, kProbeSmem, s>>>(
          L.tiles.as<uint8_t>(), L.tile_bytes, L.xsq.as<float>(), nullptr, L.coff.as<int64_t>(),
          L.cmem.as<uint32_t>(), ws.lq.as<uint8_t>(), nullptr, Dp, ws.lqsq.as<float>(), qoff,
          ws.pmem.as<uint32_t>(), item_off, C, ws.pdist.as<float>());
    HORA_LAUNCHED();
  }
  ProfScope ps("probe_select", s);
  probe_select_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(
      ws.pkeys.as<uint64_t>(), L.coff.as<int64_t>(), ws.pdist.as<float>(), ws.lqsq.as<float>(),
      L.xsqmax.as<float>(), nq, R, slack, ws.ptau.as<float>());
  HORA_LAUNCHED();
  return HORA_OK;
}

int lowp_prepare(hora_index *h, cudaStream_t s) {
  const int64_t kbe = h->precision == HORA_PREC_BF16 ? 64 : 128;
  if (round_up((int64_t)h->dim, kbe) / kbe > 2) return HORA_OK;  // exact path answers
  HORA_TRY(ensure_lowp(h, h->precision, s));
  if (probe_eligible(h)) HORA_TRY(ensure_pivots(h, *h->lowp, s));
  return HORA_OK;
}

int lowp_rerank_width(const hora_index *h, int k) {
  const int64_t kbe = h->precision == HORA_PREC_BF16 ? 64 : 128;
  if (h->metric == M_L1 || round_up((int64_t)h->dim, kbe) / kbe > 2) return 0;  // the exact path answers
  int R = h->rerank > 0 ? h->rerank
                        : (h->precision == HORA_PREC_BF16 ? std::max(2 * k, k + 64) : std::max(4 * k, k + 128));
  R = std::max(R, k);
  return (int)std::min<int64_t>(R, std::max<int64_t>(h->n, k));
}

int lowp_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                     cudaStream_t s) {
  const int prec = h->precision;
  const int64_t kbe = prec == HORA_PREC_BF16 ? 64 : 128;
  const int64_t Dp = round_up((int64_t)h->dim, kbe);
  const int nkb = (int)(Dp / kbe);
  if (h->metric == M_L1 || nkb > 2) {
    // no tensor-core form (Manhattan) or dimension beyond the resident tile:
    // the exact FP32 path answers
    int retries = 0;
    HORA_TRY(bf_topk_exact(base_view(h), h->metric, ws.q.as<float>(), ws.qnorm.as<float>(), nq, k,
                           h->cand_cap, ws, d_best, s, &retries));
    h->last_retries = retries;
    return HORA_OK;
  }
  HORA_TRY(ensure_lowp(h, prec, s));
  LowpState &L = *h->lowp;
  const int R = lowp_rerank_width(h, k);
  if (R > 4096) return fail(HORA_ECAP, "rerank width must be <= 4096");
  int cap = std::max(h->cand_cap, 2 * R);
  cap = (int)round_up(cap, 128);
  const int stages = lp_stages(nkb, prec == HORA_PREC_BF16 && h->metric == M_L2);
  const int64_t esz = prec == HORA_PREC_BF16 ? 2 : 1;

  // query copies
  HORA_TRY(ws.lq.reserve(std::max<int64_t>(nq, 1) * Dp * esz));
  HORA_TRY(ws.lerr.reserve(16));
  HORA_TRY(ws.lqsq.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  const double *qsq64 = reinterpret_cast<const double *>(ws.qnorm.as<char>() + round_up(sizeof(float) * nq, 16));
  {
    ProfScope ps("lowp_convert", s);
    if (prec == HORA_PREC_BF16) {
      to_bf16_kernel<<<ceil_div(nq * Dp, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp,
                                                            h->metric == M_COS ? qsq64 : nullptr,
                                                            ws.lq.as<__nv_bfloat16>());
    } else {
      HORA_TRY(ws.lqscale.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
      to_e4m3_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp,
                                                     ws.lq.as<uint8_t>(), ws.lqscale.as<float>());
    }
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(qsq64, nq, ws.lqsq.as<float>());
    HORA_LAUNCHED();
  }
  CUtensorMap ta;
  HORA_TRY(make_tmap(&ta, ws.lq.ptr, prec, Dp, nq, kLpBM));

  // approximate R-best lists
  HORA_TRY(ws.best.reserve(sizeof(uint64_t) * nq * R));
  HORA_TRY(ws.cand.reserve(sizeof(uint64_t) * nq * cap));
  HORA_TRY(ws.count.reserve(sizeof(uint32_t) * nq));
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(sizeof(uint32_t)));
  HORA_TRY(ws.qlist.reserve(sizeof(int) * nq));
  uint64_t *bestR = ws.best.as<uint64_t>();
  uint32_t *count = ws.count.as<uint32_t>();
  uint8_t *flags = ws.ovf_flag.as<uint8_t>();
  uint32_t *ovc = ws.ovf_counter.as<uint32_t>();
  HORA_CUDA_TRY(cudaMemsetAsync(bestR, 0xff, sizeof(uint64_t) * nq * R, s));
  HORA_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(uint32_t) * nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(flags, 0, nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(ovc, 0, sizeof(uint32_t), s));
  HORA_CUDA_TRY(cudaMemsetAsync(ws.lerr.ptr, 0, 16, s));

  LpParams p{};
  p.nq = nq;
  p.qmap = nullptr;
  p.nkb = nkb;
  p.stages = stages;
  p.xsq = L.xsq.as<float>();
  p.xscale = L.xscale.as<float>();
  p.xnorm = h->xnorm.as<float>();
  p.qsq = ws.lqsq.as<float>();
  p.qscale = ws.lqscale.as<float>();
  p.qnorm = ws.qnorm.as<float>();
  p.best = bestR;
  p.k = R;
  p.cand = ws.cand.as<uint64_t>();
  p.cap = cap;
  p.count = count;
  p.err = ws.lerr.as<int>();
  const int64_t n = h->n;
  const int64_t max_chunk = (int64_t)60000 * kLpBN * kLpMinTilesPerCta;
  // The chunked schedule for nl queries (list slots through qlist, or all;
  // tm = their query tiles): a dense first chunk, then filter chunks against
  // each query's R-th key so far.
  auto chunked = [&](const CUtensorMap &tm, int64_t nl, const int *qlist) -> int {
    LpParams c = p;
    c.nq = nl;
    c.qmap = qlist;
    c.tau0 = nullptr;
    c.dense_hits = 0;
    const int64_t c0 = std::min<int64_t>(n, std::min<int64_t>(cap, round_up(std::max(2 * R, 1024), kLpBN)));
    c.r_begin = 0;
    c.r_end = c0;
    c.tpc = lp_tiles_per_cta(nl, c0);
    HORA_TRY(launch_lp(prec, h->metric, TILE_DENSE, tm, L, c, s));
    // bestR is an intermediate list: only its R-th key (the threshold) needs its place
    HORA_TRY(launch_merge_topk(bestR, R, c.cand, count, cap, (int)c0, qlist, nl, flags, ovc, s, false));
    int64_t done = c0;
    while (done < n) {
      // each chunk at most 1.5x the rows scanned so far and at least 2,048
      // rows: a hit costs the drain more than the merge a smaller chunk adds
      // (measured on 1M x 128, R = 132)
      double grow = std::min((double)cap / (4.0 * R), 1.5);
      int64_t w = (int64_t)((double)done * std::max(grow, 1.0));
      w = std::max<int64_t>(w, (int64_t)2048);
      w = std::min<int64_t>(round_up(w, kLpBN), std::min<int64_t>(n - done, max_chunk));
      c.r_begin = done;
      c.r_end = done + w;
      // expected hits per drain thread and CTA, R x (rows per CTA / 4) / done:
      // from about 20 on, warp-converged flushes beat per-lane ones
      c.tpc = lp_tiles_per_cta(nl, w);
      c.dense_hits = (double)R * (kLpBN * c.tpc / 4) / (double)done >= 20.0;
      HORA_TRY(launch_lp(prec, h->metric, TILE_FILTER, tm, L, c, s));
      HORA_TRY(launch_merge_topk(bestR, R, c.cand, count, cap, 0, qlist, nl, flags, ovc, s, false));
      done += w;
    }
    return HORA_OK;
  };
  // gathered query tiles of the nl queries listed in ws.qlist
  auto gather = [&](int64_t nl, CUtensorMap *tg) -> int {
    HORA_TRY(ws.lqgather.reserve(nl * Dp * esz));
    gather_rows_u8_kernel<<<(unsigned)nl, 128, 0, s>>>(ws.lq.as<uint8_t>(), Dp * esz, ws.qlist.as<int>(), nl,
                                                       ws.lqgather.as<uint8_t>());
    HORA_LAUNCHED();
    return make_tmap(tg, ws.lqgather.ptr, prec, Dp, nl, kLpBM);
  };
  int *lerr = ws.lerr.as<int>();  // [0] a pipeline wait timed out, [1] short lists after the probed pass
  // (the probe kernel stages rows of at most 128 values)
  const bool probe = probe_eligible(h) && R <= kProbeMaxR && Dp <= 128;
  if (probe) {
    // one filter pass from the probed thresholds
    HORA_TRY(ensure_pivots(h, L, s));
    CUtensorMap ta16 = ta;
    if (prec == HORA_PREC_FP8) {
      // the pivot pass reads the queries in BF16
      const int64_t Dp16 = round_up((int64_t)h->dim, 64);
      HORA_TRY(ws.lq16.reserve(std::max<int64_t>(nq, 1) * Dp16 * 2));
      to_bf16_kernel<<<ceil_div(nq * Dp16, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp16, nullptr,
                                                               ws.lq16.as<__nv_bfloat16>());
      HORA_LAUNCHED();
      HORA_TRY(make_tmap(&ta16, ws.lq16.ptr, HORA_PREC_BF16, Dp16, nq, kLpBM));
    }
    HORA_TRY(probe_thresholds(h, L, prec, nq, R, Dp, ws, ta16, p, s));
    p.tau0 = ws.ptau.as<float>();
    p.dense_hits = 0;
    for (int64_t lo = 0; lo < n; lo += max_chunk) {
      p.r_begin = lo;
      p.r_end = std::min<int64_t>(n, lo + max_chunk);
      p.tpc = lp_tiles_per_cta(nq, p.r_end - p.r_begin);
      HORA_TRY(launch_lp(prec, h->metric, TILE_FILTER, ta, L, p, s));
      HORA_TRY(launch_merge_topk(bestR, R, p.cand, count, cap, 0, nullptr, nq, flags, ovc, s, false));
    }
    short_lists_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(bestR, R, nq, lerr + 1, ws.qlist.as<int>());
    HORA_LAUNCHED();
  } else {
    HORA_TRY(chunked(ta, nq, nullptr));
  }
  // exact FP32 rerank of the R candidates, then the k best; launched before
  // the host learns whether a candidate list overflowed or came out short
  // (rare), so the stream runs on without a round trip, and redone after
  HORA_TRY(ws.tmp.reserve(sizeof(uint64_t) * nq * R));
  auto finish = [&]() -> int {
    HORA_TRY(launch_rerank_exact(h->metric, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim,
                                 ws.qnorm.as<float>(), h->xnorm.as<float>(), bestR, nq, R,
                                 ws.tmp.as<uint64_t>(), s));
    HORA_CUDA_TRY(cudaMemsetAsync(d_best, 0xff, sizeof(uint64_t) * nq * k, s));
    return launch_merge_topk(d_best, k, ws.tmp.as<uint64_t>(), nullptr, R, R, nullptr, nq, flags, ovc, s);
  };
  HORA_TRY(finish());
  uint32_t h_ovc = 0;
  int hs[2] = {0, 0};
  auto status = [&]() -> int {
    HORA_CUDA_TRY(cudaMemcpyAsync(&h_ovc, ovc, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(hs, lerr, sizeof(hs), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs[0]) return fail(HORA_ETIMEDOUT, "tensor-core scan: a pipeline wait timed out");
    return HORA_OK;
  };
  HORA_TRY(status());
  h->last_probe = probe ? 1 : 0;
  bool redo = false;
  if (hs[1] > 0) {
    // lists the probed pass left short: the chunked schedule answers them
    h->last_probe = 2;
    const int64_t nl = hs[1];
    clear_lists_kernel<<<(unsigned)ceil_div(nl * R, 256), 256, 0, s>>>(bestR, R, ws.qlist.as<int>(), nl);
    HORA_LAUNCHED();
    CUtensorMap tg;
    HORA_TRY(gather(nl, &tg));
    HORA_TRY(chunked(tg, nl, ws.qlist.as<int>()));
    HORA_TRY(status());
    redo = true;
  }
  // overflow rescans over gathered query rows, against the R-th key of the
  // list so far (for a probed list that key is already at or below its
  // starting threshold)
  int rounds = 0;
  while (h_ovc > 0) {
    if (++rounds > 64) return fail(HORA_ECUDA, "candidate overflow did not converge");
    ws.h_flags.resize(nq);
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.h_flags.data(), flags, nq, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> list;
    for (int64_t q = 0; q < nq; ++q)
      if (ws.h_flags[q]) list.push_back((int)q);
    const int64_t nl = (int64_t)list.size();
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.qlist.ptr, list.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaMemsetAsync(flags, 0, nq, s));
    HORA_CUDA_TRY(cudaMemsetAsync(ovc, 0, sizeof(uint32_t), s));
    CUtensorMap tg;
    HORA_TRY(gather(nl, &tg));
    LpParams r = p;
    r.nq = nl;
    r.qmap = ws.qlist.as<int>();
    r.tau0 = nullptr;
    r.dense_hits = 0;
    for (int64_t lo = 0; lo < n; lo += max_chunk) {
      r.r_begin = lo;
      r.r_end = std::min<int64_t>(n, lo + max_chunk);
      r.tpc = lp_tiles_per_cta(nl, r.r_end - r.r_begin);
      HORA_TRY(launch_lp(prec, h->metric, TILE_FILTER, tg, L, r, s));
      HORA_TRY(launch_merge_topk(bestR, R, p.cand, count, cap, 0, ws.qlist.as<int>(), nl, flags, ovc, s));
    }
    HORA_TRY(status());
    redo = true;
  }
  h->last_retries = rounds;
  if (redo) HORA_TRY(finish());
  return HORA_OK;
}

// ---- exact search certified on the tensor cores ------------------------------------
// Exact FP32 Euclidean search (the reference's result, distances bit for
// bit) on at least kProbeMinRows rows with the BF16 scan as a certified
// filter.  For every row x and query q the scan's value s(q, x) = |q|^2 -
// 2 (<q~, x~> - |x|^2 / 2) and the reference's sequential f32 sum r(q, x)
// differ by at most eps(q):
//   <q~, x~> - <q, x> = <q~, x~ - x> + <q~ - q, x>, so by Cauchy-Schwarz
//   |.| <= |q~| max|x - x~| + |q - q~| max|x|               (term A)
//   the tensor core's FP32 accumulation of Dp + 16 exact products,
//   bounded generously by (Dp + 16) 2^-22 (|q~| max|x~| + max|x|^2 / 2)  (B)
//   the f32 roundings of |x|^2 / 2, |q|^2 and the final FMA            (C)
//   the reference's own f32 sum, (dim + 4) 2^-23 (|q| + max|x|)^2     (E)
//   eps = 2 A + 2 B + C + E.
// The probe (probe_dist_kernel, same products, another f32 order, within
// delta = 1e-4 (|q|^2 + max|x|^2) of the scan) puts a query's k-th smallest
// probe value t among its pivot cluster's members.  k rows then have r <= t
// + delta + eps, so the exact k-th distance is at most that, and every row
// of the exact top k has s <= t + delta + 2 eps: the filter pass from that
// threshold keeps them all.  The kept rows are rescored exactly (reference
// op order) and the k best returned.  A query whose cluster has fewer than k
// members, or whose kept rows overflow the candidate capacity, is answered
// by the CUDA-core exact scan instead; either way the result is exact.

// 2 eps(q) per query (rounded up), from the staged f32 query rows.
__global__ void exact_tc_slack_kernel(const float *Q, int64_t nq, int64_t ld, int64_t dim, int64_t Dp,
                                      const double *qsq64, const float *dxmax, const float *xsqmax,
                                      float *slack) {
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  double sb = 0.0, sd = 0.0;
  for (int64_t t = lane; t < dim; t += 32) {
    const float x = Q[q * ld + t];
    const double b = (double)__bfloat162float(__float2bfloat16_rn(x));
    sb += b * b;
    sd += ((double)x - b) * ((double)x - b);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
    sd += __shfl_xor_sync(0xffffffffu, sd, o);
  }
  if (lane) return;
  const double qb = sqrt(sb) * (1.0 + 0x1p-40), dq = sqrt(sd) * (1.0 + 0x1p-40);
  const double qsq = qsq64[q], qn = sqrt(qsq);
  const double xsq = (double)*xsqmax * (1.0 + 0x1p-22), xn = sqrt(xsq);
  const double dx = (double)*dxmax;
  const double xb = xn * (1.0 + 0x1p-8) + dx;  // |bf16(x)| <= |x| + |x - bf16(x)|
  const double A = qb * dx + dq * xn;
  const double B = (double)(Dp + 16) * 0x1p-22 * (qb * xb + 0.5 * xsq);
  const double Cr = 0x1p-22 * (qsq + 2.0 * qb * xb + xsq);
  const double E = (double)(dim + 4) * 0x1p-23 * (qn + xn) * (qn + xn);
  const double eps = 2.0 * A + 2.0 * B + Cr + E;
  slack[q] = nextafterf((float)(2.0 * eps * (1.0 + 0x1p-10)), INFINITY);
}

// Queries the certified pass cannot answer: fewer than k rows kept (no
// valid probe) or more than the capacity (overflow).
__global__ void exact_tc_fallback_kernel(const uint32_t *count, int64_t nq, int k, int cap, int *n, int *list) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq && (count[q] < (uint32_t)k || count[q] > (uint32_t)cap)) list[atomicAdd(n, 1)] = (int)q;
}

__global__ void gather_rows_f32_kernel(const float *src, int64_t ld, const int *list, int64_t nl, float *dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl * ld) dst[i] = src[(int64_t)list[i / ld] * ld + (i % ld)];
}

__global__ void scatter_keys_kernel(const uint64_t *src, int k, const int *list, int64_t nl, uint64_t *dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl * k) dst[(int64_t)list[i / k] * k + (i % k)] = src[i];
}

bool exact_tc_eligible(const hora_index *h, int k) {
  return h->exact_tc && h->precision == HORA_PREC_FP32 && h->metric == M_L2 && h->n >= kProbeMinRows &&
         round_up((int64_t)h->dim, 64) / 64 <= 2 && k <= kExactTcMaxK;
}

int exact_tc_prepare(hora_index *h, cudaStream_t s) {
  HORA_TRY(ensure_lowp(h, HORA_PREC_BF16, s));
  return ensure_pivots(h, *h->lowp, s);
}

int exact_tc_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                         cudaStream_t s) {
  const int64_t Dp = round_up((int64_t)h->dim, 64);
  const int nkb = (int)(Dp / 64);
  HORA_TRY(ensure_lowp(h, HORA_PREC_BF16, s));
  LowpState &L = *h->lowp;
  HORA_TRY(ensure_pivots(h, L, s));
  const int cap = (int)round_up(std::max(h->cand_cap, 2 * k), 128);
  const int stages = lp_stages(nkb, true);
  // BF16 queries, their f32 squared norms and the certified slack
  HORA_TRY(ws.lq.reserve(std::max<int64_t>(nq, 1) * Dp * 2));
  HORA_TRY(ws.lerr.reserve(16));
  HORA_TRY(ws.lqsq.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  HORA_TRY(ws.xslack.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  const double *qsq64 = reinterpret_cast<const double *>(ws.qnorm.as<char>() + round_up(sizeof(float) * nq, 16));
  {
    ProfScope ps("lowp_convert", s);
    to_bf16_kernel<<<ceil_div(nq * Dp, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, nullptr,
                                                          ws.lq.as<__nv_bfloat16>());
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(qsq64, nq, ws.lqsq.as<float>());
    HORA_LAUNCHED();
    exact_tc_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, qsq64,
                                                          L.dxmax.as<float>(), L.xsqmax.as<float>(),
                                                          ws.xslack.as<float>());
    HORA_LAUNCHED();
  }
  CUtensorMap ta;
  HORA_TRY(make_tmap(&ta, ws.lq.ptr, HORA_PREC_BF16, Dp, nq, kLpBM));
  HORA_TRY(ws.xempty.reserve(sizeof(uint64_t) * std::max<int64_t>(nq, 1)));
  HORA_TRY(ws.cand.reserve(sizeof(uint64_t) * nq * cap));
  HORA_TRY(ws.count.reserve(sizeof(uint32_t) * nq));
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(sizeof(uint32_t)));
  HORA_TRY(ws.xlist.reserve(sizeof(int) * std::max<int64_t>(nq, 1)));
  uint32_t *count = ws.count.as<uint32_t>();
  uint8_t *flags = ws.ovf_flag.as<uint8_t>();
  uint32_t *ovc = ws.ovf_counter.as<uint32_t>();
  int *lerr = ws.lerr.as<int>();  // [0] a pipeline wait timed out, [1] fallback queries
  HORA_CUDA_TRY(cudaMemsetAsync(ws.xempty.ptr, 0xff, sizeof(uint64_t) * nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(uint32_t) * nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(flags, 0, nq, s));
  HORA_CUDA_TRY(cudaMemsetAsync(ovc, 0, sizeof(uint32_t), s));
  HORA_CUDA_TRY(cudaMemsetAsync(ws.lerr.ptr, 0, 16, s));
  LpParams p{};
  p.nq = nq;
  p.nkb = nkb;
  p.stages = stages;
  p.xsq = L.xsq.as<float>();
  p.xnorm = h->xnorm.as<float>();
  p.qsq = ws.lqsq.as<float>();
  p.qnorm = ws.qnorm.as<float>();
  p.best = ws.xempty.as<uint64_t>();  // no list: the probed threshold alone decides
  p.k = 1;
  p.cand = ws.cand.as<uint64_t>();
  p.cap = cap;
  p.count = count;
  p.err = lerr;
  HORA_TRY(probe_thresholds(h, L, HORA_PREC_BF16, nq, k, Dp, ws, ta, p, s, ws.xslack.as<float>()));
  p.tau0 = ws.ptau.as<float>();
  const int64_t n = h->n;
  const int64_t max_chunk = (int64_t)60000 * kLpBN * kLpMinTilesPerCta;
  for (int64_t lo = 0; lo < n; lo += max_chunk) {
    p.r_begin = lo;
    p.r_end = std::min<int64_t>(n, lo + max_chunk);
    p.tpc = lp_tiles_per_cta(nq, p.r_end - p.r_begin);
    HORA_TRY(launch_lp(HORA_PREC_BF16, M_L2, TILE_FILTER, ta, L, p, s));
  }
  // the queries the pass cannot answer (read before the merge, which
  // consumes the counts), every kept row rescored exactly, then the k best
  exact_tc_fallback_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(count, nq, k, cap, lerr + 1,
                                                                     ws.xlist.as<int>());
  HORA_LAUNCHED();
  HORA_TRY(launch_rerank_exact(M_L2, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim, nullptr, nullptr,
                               p.cand, nq, cap, p.cand, s, count));
  HORA_CUDA_TRY(cudaMemsetAsync(d_best, 0xff, sizeof(uint64_t) * nq * k, s));
  HORA_TRY(launch_merge_topk(d_best, k, p.cand, count, cap, 0, nullptr, nq, flags, ovc, s));
  int hs[2] = {0, 0};
  HORA_CUDA_TRY(cudaMemcpyAsync(hs, lerr, sizeof(hs), cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  if (hs[0]) return fail(HORA_ETIMEDOUT, "tensor-core scan: a pipeline wait timed out");
  h->last_probe = 1;
  h->last_retries = 0;
  h->last_fallback = hs[1];
  if (hs[1] > 0) {
    // the queries the certified pass could not answer: the CUDA-core scan
    h->last_probe = 2;
    const int64_t nl = hs[1];
    HORA_TRY(ws.xq.reserve(sizeof(float) * nl * h->ld));
    HORA_TRY(ws.xkeys.reserve(sizeof(uint64_t) * nl * k));
    gather_rows_f32_kernel<<<ceil_div(nl * (int64_t)h->ld, 256), 256, 0, s>>>(ws.q.as<float>(), h->ld,
                                                                             ws.xlist.as<int>(), nl,
                                                                             ws.xq.as<float>());
    HORA_LAUNCHED();
    int retries = 0;
    HORA_TRY(bf_topk_exact(base_view(h), M_L2, ws.xq.as<float>(), nullptr, nl, k, h->cand_cap, ws,
                           ws.xkeys.as<uint64_t>(), s, &retries));
    scatter_keys_kernel<<<ceil_div(nl * (int64_t)k, 256), 256, 0, s>>>(ws.xkeys.as<uint64_t>(), k,
                                                                      ws.xlist.as<int>(), nl, d_best);
    HORA_LAUNCHED();
    h->last_retries = retries;
  }
  return HORA_OK;
}

}  // namespace hora
