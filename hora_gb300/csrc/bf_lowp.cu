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
// Base tiles per CTA: up to 128 (32,768 rows) amortises the CTA prologue
// and epilogue, which no other CTA overlaps at one CTA per SM (the probed
// pass over 1M rows at 10k queries: 1.98 ms at 32, 1.88 at 64, 1.84 at 128,
// 1.87 at 256); a launch with few query blocks takes fewer, down to 8, so
// that it still spreads over every SM (see lp_tiles_per_cta).
constexpr int kLpTilesPerCta = 128;
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
// Base rows gathered into a tile image of the base's layout and precision
// (converted by the same kernels, so every value equals the base image's),
// with the per-row values the scan's drain reads (exact squared norms, e4m3
// scales, norms); padding rows are zero.
struct RowImage {
  DevBuf tiles, xsq, xscale, xnorm, gmeta;
  int64_t rows = 0;  // a multiple of the tile
};

struct LowpState {
  int prec = 0, metric = 0;
  int64_t n = 0, Dp = 0;
  DevBuf tiles;    // ceil(n / 256) x tile_bytes
  int64_t tile_bytes = 0;
  DevBuf xsq;      // n f32 exact squared norms
  DevBuf xscale;   // n f32 (e4m3 per-row scale)
  DevBuf gmeta;    // e4m3: per 32 rows the filter's bound inputs (see group_meta_kernel)
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
  // the members' image: cluster c's first min(members, kProbeMaxMembers)
  // rows from image row moff[c] (a multiple of the tile)
  RowImage members;
  DevBuf moff;
  // the sample image: base rows floor(frac(j phi) n), j = 1, 2, ... (any
  // prefix spread over the base), for wide R-best lists
  RowImage sample;
  // BF16 Euclidean and DotProduct: the largest |x - bf16(x)| over the rows
  // (1 f32, rounded up), the rows' share of the certified error bounds
  DevBuf dxmax;
  // BF16 Euclidean: each row's |x - bf16(x)| (n f32, rounded up), for the
  // per-row window of the certified exact search
  DevBuf dxrow;
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
  // work items instead of the (query block, row chunk) grid: CTA b takes
  // items[b] = {first query row, query rows, first image row (a multiple of
  // the tile), columns}, for b < *n_items
  const int4 *items;
  const int *n_items;
  // TILE_DIST: distances out_dist[query row * ldo + column]
  float *out_dist;
  int64_t ldo;
  // FP8 filter: per 32 image rows {min |x|^2, min scale, max scale, 0}, or
  // null (see group_meta_kernel)
  const float4 *gmeta;
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

// TILE_DIST: a slice's 32 distances to the query's output row (orow is
// indexed by image row; 16-byte stores for a whole slice: the row's
// columns start a multiple of 32 into a 16-byte aligned row).
template <int MT, bool RAW>
__device__ __forceinline__ void store_dist(const uint32_t (&v)[32], const DrainCtx &c, float *orow) {
  float *o = orow + c.rt;
  if (c.rt + 32 <= c.r_end) {
#pragma unroll
    for (int j = 0; j < 32; j += 4)
      *reinterpret_cast<float4 *>(o + j) =
          make_float4(drain_dist<MT, TILE_DIST, RAW>(v[j], c.qa), drain_dist<MT, TILE_DIST, RAW>(v[j + 1], c.qa),
                      drain_dist<MT, TILE_DIST, RAW>(v[j + 2], c.qa), drain_dist<MT, TILE_DIST, RAW>(v[j + 3], c.qa));
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (c.rt + j < c.r_end) o[j] = drain_dist<MT, TILE_DIST, RAW>(v[j], c.qa);
  }
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
  int64_t q0, row0, r_end;
  int T, nqv;  // tiles, query rows of the block
  if (p.items) {
    if ((int)blockIdx.x >= *p.n_items) return;  // the grid is an upper bound
    const int4 it = p.items[blockIdx.x];
    q0 = it.x;
    nqv = it.y;
    row0 = it.z;
    r_end = row0 + it.w;
    T = (it.w + kLpBN - 1) / kLpBN;
  } else {
    q0 = (int64_t)blockIdx.x * kLpBM;
    nqv = kLpBM;
    row0 = p.r_begin + (int64_t)blockIdx.y * kLpBN * p.tpc;
    r_end = p.r_end;
    T = (int)std::min<int64_t>(p.tpc, (r_end - row0 + kLpBN - 1) / kLpBN);
  }

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
      tc::mbar_init(acc_empty + b, kLpEpiThreads / 32);  // one arrival per drain warp
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
    // (its waits poll instead of sleeping in try_wait: the thread's wake-up
    // after a slot fills or an accumulator frees gates the tensor pipe)
    if (tc::elect_one()) {
      constexpr uint32_t idesc = tc::idesc_f32acc(PREC == HORA_PREC_BF16 ? 1u : 0u, kLpBM, kLpBN);
      bool ok = tc::mbar_wait(a_full, 0, abort);
      const bool rest = nkb > 1 || FOLD;  // a second half exists
      for (int t = 0; ok && t < T; ++t) {
        const int s = t % S, j = t / S, b = t % kLpNB, jb = t / kLpNB;
        if (!tc::mbar_wait_poll(full + s, j & 1, abort)) break;
        if (jb > 0 && !tc::mbar_wait_poll(acc_empty + b, (jb - 1) & 1, abort)) break;
        tc::fence_after_sync();
        const uint32_t d = tmem + (uint32_t)(b * kLpBN);
        uint8_t *st = sB + (size_t)s * stage_bytes;
        bool ok2 = true;
        for (int kb = 0; kb < nkb; ++kb) {
          if (kb == 1) {
            // K block 0 read: its half of the stage may be refilled
            tc::mma_commit(empty + s);
            if (!tc::mbar_wait_poll(full2 + s, j & 1, abort)) {
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
            if (!tc::mbar_wait_poll(full2 + s, j & 1, abort)) break;
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
    const int64_t qid = qrow < p.nq && m < nqv ? (p.qmap ? p.qmap[qrow] : qrow) : -1;
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
    DrainCtx c{p.cand, p.count, hbuf + (threadIdx.x - 64), qid, 0, p.r_begin, r_end, p.cap, qa, tau_d, tau_r};
    // TILE_DIST: column = image row - the item's first row (work items) or
    // the launch's first row
    float *orow = MODE == TILE_DIST && qid >= 0 ? p.out_dist + qrow * p.ldo - (p.items ? row0 : p.r_begin) : nullptr;
    int nb = 0;  // keys staged in this thread's column
    for (int t = 0; t < T; ++t) {
      const int b = t % kLpNB, jb = t / kLpNB;
      // e4m3 filter: this warp's two slices' bound inputs, loaded while the
      // MMAs of the tile run
      static_assert(kLpSlices == 2, "two slices per drain warp and tile");
      float4 gm0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), gm1 = gm0;
      if (!FAST && MODE == TILE_FILTER && (MT == M_L2 || MT == M_IP) && p.gmeta) {
        const int64_t g0 = (row0 + (int64_t)t * kLpBN + h * kLpSlices * 32) >> 5;
        gm0 = __ldg(p.gmeta + g0);
        gm1 = __ldg(p.gmeta + g0 + 1);
      }
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
      uint32_t v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(b * kLpBN + (h * kLpSlices + sl) * 32), v);
      tc::tmem_ld_wait();
      if (sl == kLpSlices - 1) {
        // every lane's loads are complete (tcgen05.wait::ld): one arrival
        // for the warp instead of one per thread on the same barrier word
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(acc_empty + b);
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
        } else if constexpr (MODE == TILE_DIST) {
          if (qid >= 0) store_dist<MT, true>(v, c, orow);
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
      if constexpr (MODE == TILE_FILTER && (MT == M_L2 || MT == M_IP)) {
        // e4m3 filter on the raw accumulators: from the slice's bound inputs
        // (smallest squared norm, scale range of its 32 rows) an accumulator
        // threshold th such that a column whose key clears tau has acc >= th
        // (Euclidean: qsq + |x|^2 - 2 qs xs acc <= tau needs 2 qs max(xs) acc
        // >= qsq + min|x|^2 - tau) or acc <= th (DotProduct: qs xs acc <=
        // tau), loosened by a relative 1e-5 for the f32 roundings.  When the
        // slice's extreme clears no lane's threshold, the warp skips the
        // per-column pass; the decision is a warp vote, because that pass
        // shuffles across all 32 lanes.
        if (p.gmeta) {
          const float4 gm = sl == 0 ? gm0 : gm1;
          float th;
          if (MT == M_L2) {
            const float slack = 1e-5f * (fabsf(qa) + fabsf(gm.x) + fabsf(tau_d));
            th = ((qa + gm.x) - tau_d - slack) / (2.0f * qs * gm.z);
            th = th > 0.0f ? th * (1.0f - 1e-5f) : -__int_as_float(0x7f800000);  // else every column
          } else {
            th = tau_d / (qs * (tau_d >= 0.0f ? gm.y : gm.z));
            th = th + 1e-5f * fabsf(th) + 1e-30f;
          }
          bool maybe = false;
          if (qid >= 0) {
            const float ext = slice_extreme<MT == M_IP>(v);
            maybe = MT == M_L2 ? ext >= th : ext <= th;
          }
          if (!__any_sync(0xffffffffu, maybe)) continue;
        }
      }
      // generic forms: this lane's row factor, broadcast by shuffle below
      float xa = 0.0f, xs = 1.0f;
      {
        const int64_t r = c.rt + lane;
        const float *va = MT == M_L2 ? p.xsq : (MT == M_COS ? p.xnorm : nullptr);
        if (va) xa = r < r_end ? __ldg(va + r) : 0.0f;
        if (PREC == HORA_PREC_FP8) xs = r < r_end ? __ldg(p.xscale + r) : 0.0f;
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
      if constexpr (MODE == TILE_DIST) {
        if (qid >= 0) store_dist<MT, false>(v, c, orow);
      } else {
        if (MODE == TILE_DENSE) hits = 0xffffffffu;
        if (qid >= 0 && hits) drain_mask<MT, MODE, false>(v, hits, c, nb);
      }
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
__global__ void bf16_residual_max_kernel(const float *X, int64_t n, int64_t ld, int64_t dim, unsigned *out,
                                         float *row_out = nullptr) {
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
  const float e = nextafterf((float)sqrt(acc), INFINITY);
  if (lane == 0) {
    atomicMax(out, __float_as_uint(e));
    if (row_out) row_out[r] = e;
  }
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

// ---- starting thresholds ------------------------------------------------------------
// With a threshold that starts at the R-th key of the rows scanned so far,
// the chunked schedule keeps about R x ln(n / first chunk) rows per query
// (~1,500 on 1M rows, R = 132), and the drain's hit handling is the largest
// cost of the scan after the MMAs.  A base of at least kProbeMinRows rows
// therefore gives every query a starting threshold before one filter pass
// over the whole base.  A query that kept at least R rows has its R-best set
// complete: R rows at or below the threshold put its R-th key there, and
// every key up to that one was kept.  A query that kept fewer is answered
// again by the chunked schedule.  So the threshold only decides the cost.
//
// Up to R = kProbeClusterMaxR the threshold is a bound.  The base keeps
// ~n / 1,024 pivot clusters (a few Lloyd steps from evenly spaced rows;
// clusters below kProbeMinCluster members dissolved, empty ones dropped).
// Every query goes to its nearest pivot in the index's own metric (a BF16
// pass over the pivots' image: Euclidean with the norm folded in,
// CosineSimilarity on unit pivots, DotProduct ascending +<q, c>) and is
// scored against up to kProbeMaxMembers rows of that cluster by the scan
// kernel itself: the members' rows are kept as a second tile image (each
// cluster's first kProbeMaxMembers members, every cluster starting on a
// tile, converted exactly as the base's image), the queries are gathered in
// pivot order, and one CTA per (pivot, up to 128 of its queries) writes the
// keys of those members (TILE_DIST): the same operands, MMAs and key formula
// as the scan.  The threshold is the R-th of those keys plus a bound
// covering any difference in summation order; a cluster holds at least
// kProbeMinCluster >= R rows, so no list comes out short.
//
// Wider lists (up to kProbeMaxR) take a sampled threshold instead
// (sample_threshold): the R best rows of a large base are often thin tails
// of many clusters, so the R-th key of one cluster's members lies far above
// the base's R-th key.
constexpr int64_t kProbeRowsPerPivot = 1024;
constexpr int64_t kProbeMinRows = 65536;
constexpr int kProbeMaxMembers = 1024;  // members of a cluster a query is scored against
constexpr int kProbeClusterMaxR = 256;  // widest R-best list with a cluster threshold
constexpr int kProbeMaxR = 4096;        // widest R-best list with a sampled threshold
constexpr int kExactTcMaxK = 256;       // largest k of the certified exact search
constexpr int kProbeMinCluster = 256;   // smaller clusters are dissolved at the end
constexpr int kProbeReseed = 128;       // Lloyd steps re-seed clusters below this
constexpr int kProbeLloyd = 6;
constexpr int64_t kProbeSampleRows = 262144;  // rows of the sample image at most
static_assert(kProbeMinCluster >= kProbeClusterMaxR, "a cluster must hold the widest clustered R-best list");

// Row i of the members' image: the base row of member i - moff[c] of the
// cluster c whose image rows hold i, or none (0xffffffff) past its first
// min(members, kProbeMaxMembers) members.
__global__ void member_rows_kernel(const int64_t *coff, const uint32_t *cmem, const int64_t *moff, int C,
                                   int64_t nimg, uint32_t *mrow) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nimg) return;
  int lo = 0, hi = C;  // the last c with moff[c] <= i
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (moff[mid] <= i) lo = mid; else hi = mid;
  }
  const int64_t j = i - moff[lo], cnt = coff[lo + 1] - coff[lo];
  mrow[i] = j < cnt && j < kProbeMaxMembers ? cmem[coff[lo] + j] : 0xffffffffu;
}

// Sample image rows: j < m holds base row floor(frac((j + 1) phi) n) (phi
// the golden ratio: every prefix is spread evenly over the rows), the rest
// padding.
__global__ void sample_rows_kernel(int64_t n, int64_t m, int64_t ns, uint32_t *rowmap) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  if (j >= m) {
    rowmap[j] = 0xffffffffu;
    return;
  }
  const double f = (double)(j + 1) * 0.6180339887498949;
  const int64_t r = (int64_t)((f - floor(f)) * (double)n);
  rowmap[j] = (uint32_t)(r < n ? r : n - 1);
}

// FP32 rows (pitch ld) and per-row values of the members' image rows (zero
// for padding rows); any output may be null.
__global__ void gather_members_kernel(const float *X, int64_t ld, const uint32_t *mrow, int64_t nimg,
                                      const double *sq64, const float *xsq, const float *xnorm, float *rows,
                                      double *sq64_out, float *xsq_out, float *xnorm_out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nimg * ld) return;
  const int64_t r = i / ld, t = i % ld;
  const uint32_t b = mrow[r];
  rows[i] = b == 0xffffffffu ? 0.0f : X[(int64_t)b * ld + t];
  if (t == 0) {
    if (sq64_out) sq64_out[r] = b == 0xffffffffu ? 0.0 : sq64[b];
    if (xsq_out) xsq_out[r] = b == 0xffffffffu ? 0.0f : xsq[b];
    if (xnorm_out) xnorm_out[r] = b == 0xffffffffu ? 0.0f : xnorm[b];
  }
}

// Probe work items, one CTA of 1,024 threads (C <= 4,096): pivot c with
// pairs qoff[c]..qoff[c+1] (in pivot order) owns ceil(pairs / 128) items
// {first pair, pairs, first image row moff[c], min(members, kProbeMaxMembers)}.
__global__ void probe_items_kernel(const int64_t *qoff, const int64_t *coff, const int64_t *moff, int C,
                                   int4 *items, int *n_items) {
  __shared__ int part[1024];
  const int t = threadIdx.x, per = (C + 1023) / 1024;
  const int lo = min(C, t * per), hi = min(C, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += (int)((qoff[c + 1] - qoff[c] + kLpBM - 1) / kLpBM);
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int i = 0; i < 1024; ++i) {
      const int v = part[i];
      part[i] = run;
      run += v;
    }
    *n_items = run;
  }
  __syncthreads();
  int run = part[t];
  for (int c = lo; c < hi; ++c) {
    const int64_t cnt = coff[c + 1] - coff[c];
    const int cols = (int)(cnt < kProbeMaxMembers ? cnt : kProbeMaxMembers);
    for (int64_t q = qoff[c]; q < qoff[c + 1]; q += kLpBM) {
      const int nb = (int)(qoff[c + 1] - q < kLpBM ? qoff[c + 1] - q : kLpBM);
      items[run++] = make_int4((int)q, nb, (int)moff[c], cols);
    }
  }
}

// The inverse of a permutation: pos_of[perm[i]] = i.
__global__ void inverse_kernel(const uint32_t *perm, int64_t n, uint32_t *pos_of) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pos_of[perm[i]] = (uint32_t)i;
}

// The summation-order bound added to a probed threshold.  The probe and the
// scan add the same exact products (BF16 x BF16, or e4m3 x e4m3 before the
// scales) in f32 in different orders; each sum is within (Dp + 16) 2^-24 of
// the sum of the products' magnitudes.  Euclidean (norm folded: <= |q||x| +
// |x|^2 / 2 <= |q|^2 / 2 + max|x|^2) and DotProduct (<= |q||x|) keys are 2 x
// or 1 x such a sum: they differ by less than 3.5e-5 (|q|^2 + max|x|^2),
// and 1e-4 of it is taken.  CosineSimilarity keys are a sum of unit rows'
// products (or one divided by |q||x|): at most 1 in magnitude, 2e-4 taken.
__device__ __forceinline__ float probe_bound(int metric, float qsq, float xsqmax) {
  return metric == M_COS ? 2e-4f : 1e-4f * (qsq + xsqmax);
}

// The probed threshold from the upper bound a of the R-th key (ordered
// bits): the bound above, and for the certified exact search its slack (and
// a relative 2^-20 against the rounding of these f32 additions).
__device__ __forceinline__ float probe_tau(uint32_t a, int metric, float qsq, float xsqmax, const float *slack,
                                           int64_t q) {
  float t = ord2f(a) + probe_bound(metric, qsq, xsqmax);
  if (slack) t = t + slack[q] + 0x1p-20f * fabsf(t + slack[q]);
  return t;
}

// The descent stops kSelectSkip bits short of the R-th value's ordered
// encoding and rounds up: an upper bound within 2^-(23 - kSelectSkip) of
// it, which is all a threshold needs.
constexpr int kSelectSkip = 12;

// Members of the cluster of pivot key pk scored for a query (0 for an
// empty key).
__device__ __forceinline__ int probe_members(uint64_t pk, const int64_t *coff, int C) {
  const uint32_t c = key_row(pk);
  if (pk == kEmptyKey || c >= (uint32_t)C) return 0;
  const int64_t L = coff[c + 1] - coff[c];
  return (int)(L < kProbeMaxMembers ? L : kProbeMaxMembers);
}

// One cluster per query, one warp per query: the R-th smallest probe key
// by a bitwise descent over the ordered encoding, plus probe_bound.  The
// keys of pair (q, p) are row pos_of[q P + p] of pdist.  A cluster with
// fewer than R members gives -FLT_MAX: the scan keeps nothing and the query
// is rescheduled.
__global__ void probe_select_kernel(const uint64_t *pkeys, const int64_t *coff, int C, const float *pdist,
                                    const uint32_t *pos_of, const float *qsq, const float *xsqmax, int metric,
                                    int64_t nq, int R, const float *slack, float *tau) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const int L = probe_members(pkeys[q], coff, C);
  if (L < R) {
    if (lane == 0) tau[q] = -FLT_MAX;
    return;
  }
  const float *pq = pdist + (int64_t)pos_of[q] * kProbeMaxMembers;
  uint32_t v[kProbeMaxMembers / 32];
#pragma unroll
  for (int i = 0; i < kProbeMaxMembers / 32; ++i) {
    const int m = lane + 32 * i;
    v[i] = m < L ? f2ord(pq[m]) : 0xffffffffu;
  }
  // the largest a with fewer than R values below it is the R-th smallest;
  // the bits above the highest one in which the members' values differ are
  // theirs in common (a descent through them would take exactly those: a
  // set bit leaves no value below, a clear one all L >= R), so it starts
  // below them
  uint32_t lo = 0xffffffffu, hi = 0u;
#pragma unroll
  for (int i = 0; i < kProbeMaxMembers / 32; ++i) {
    if (lane + 32 * i < L) {
      lo = min(lo, v[i]);
      hi = max(hi, v[i]);
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  const int top = 31 - __clz((int)(lo ^ hi));  // -1 when every value is equal
  uint32_t a = top < 0 ? lo : top >= 31 ? 0u : lo & ~((2u << top) - 1u);
  for (int b = top; b >= kSelectSkip; --b) {
    const uint32_t tt = a | (1u << b);
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < kProbeMaxMembers / 32; ++i) cnt += v[i] < tt;
#pragma unroll
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (cnt < R) a = tt;
  }
  if (lane == 0) tau[q] = probe_tau(a | ((1u << kSelectSkip) - 1), metric, qsq[q], *xsqmax, slack, q);
}

// A query left without a pivot key (no finite distance to any pivot) takes
// the last pivot: any cluster gives a valid threshold, and every query is
// bucketed, so the buckets order all of them.
__global__ void fill_empty_pivot_kernel(uint64_t *pk, int64_t n, int C) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && pk[i] == kEmptyKey) pk[i] = make_key(__int_as_float(0x7f800000), (uint32_t)(C - 1));
}

// A query's threshold from the j-th key of its sorted sample list (first:
// set, +inf when the list is shorter; else lowered when the key exists).
__global__ void sample_tau_kernel(const uint64_t *best, int rs, int j, int64_t nq, bool first, float *tau) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t kk = best[q * rs + (j - 1)];
  const float t = kk == kEmptyKey ? __int_as_float(0x7f800000) : key_dist(kk);
  tau[q] = first ? t : fminf(tau[q], t);
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

// 2 eps(q) per query (rounded up) for the windowed rerank of a BF16 list,
// eps(q) bounding |scan key - exact distance| for every row (Q the staged
// f32 query rows):
//   DotProduct (key +<q~, x~> against the reference's sequential f32 sum):
//   |<q~, x~> - <q, x>| <= |q~| max|x - x~| + |q - q~| max|x|         (A)
//   the tensor core's f32 accumulation of Dp exact products,
//   generously (Dp + 16) 2^-22 |q~| max|x~|                            (B)
//   the reference's own sum, (dim + 4) 2^-23 |q| max|x|                 (E)
//   CosineSimilarity (key -<q^, x^> on BF16 unit rows against the
//   reference's f32 -ab / (sqrt(aa) sqrt(bb))): each unit row is rounded
//   to f32 then BF16 (relative 2^-9 + 2^-24 per element), so
//   |<q^, x^> - <u, v>| <= 2^-8 (1 + 2^-8) + 2^-8 for the exact unit
//   rows u, v                                                           (A)
//   (Dp + 16) 2^-22 (1 + 2^-8)^2 for the accumulation                   (B)
//   and (2 dim + 8) 2^-24 for the reference's sums, roots and division  (E)
//   (zero rows: both keys are 0).
__global__ void rerank_slack_kernel(const float *Q, int64_t nq, int64_t ld, int64_t dim, int64_t Dp, int metric,
                                    const double *qsq64, const float *dxmax, const float *xsqmax, float *slack) {
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  double eps;
  if (metric == M_COS) {
    if (lane) return;
    const double u = 0x1p-8;
    eps = u * (1.0 + u) + u + (double)(Dp + 16) * 0x1p-22 * (1.0 + u) * (1.0 + u) + (double)(2 * dim + 8) * 0x1p-24;
  } else {
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
    const double qn = sqrt(qsq64[q]) * (1.0 + 0x1p-40);
    const double xn = sqrt((double)*xsqmax * (1.0 + 0x1p-22)), dx = (double)*dxmax;
    const double xb = xn * (1.0 + 0x1p-8) + dx;
    eps = qb * dx + dq * xn + (double)(Dp + 16) * 0x1p-22 * qb * xb + (double)(dim + 4) * 0x1p-23 * qn * xn;
  }
  slack[q] = nextafterf((float)(2.0 * eps * (1.0 + 0x1p-10)), INFINITY);
}

// The windowed rerank's candidates: query q's keys (R slots of best) whose
// distance is at most the k-th smallest key's plus slack[q] (and a relative
// 2^-20 against the rounding of that f32 addition), moved to the front of
// its R slots of out, their number to count[q].  One warp per query.
__global__ void rerank_window_kernel(const uint64_t *best, int R, const uint64_t *kth, int k, const float *slack,
                                     int64_t nq, uint64_t *out, uint32_t *count) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const uint64_t tk = kth[q * k + (k - 1)];
  float w = __int_as_float(0x7f800000);
  if (tk != kEmptyKey) {
    const float t = key_dist(tk) + slack[q];
    w = t + 0x1p-20f * fabsf(t);
  }
  uint32_t n = 0;
  for (int i0 = 0; i0 < R; i0 += 32) {
    const int i = i0 + lane;
    const uint64_t key = i < R ? best[q * R + i] : kEmptyKey;
    const bool keep = key != kEmptyKey && key_dist(key) <= w;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) out[q * R + n + __popc(m & ((1u << lane) - 1u))] = key;
    n += __popc(m);
  }
  if (lane == 0) count[q] = n;
}

// Empties the R-best lists of the listed queries.
__global__ void clear_lists_kernel(uint64_t *best, int R, const int *list, int64_t nl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl * R) best[(int64_t)list[i / R] * R + (i % R)] = kEmptyKey;
}

// e4m3 filter bound inputs per group of 32 rows, for ngroups groups (every
// group of the image's tiles; rows past n excluded, a group without rows
// gets {+inf, +inf, 0, 0}): {min |x|^2, min scale, max scale, 0}.  A column's Euclidean distance
// qsq + |x|^2 - 2 qscale xscale acc is at least qsq + min|x|^2 - 2 qscale
// (max scale if the slice's largest acc is positive, else min scale) x that
// acc; a DotProduct key qscale xscale acc is at least qscale (max scale if
// the smallest acc is negative, else min scale) x that acc.
__global__ void group_meta_kernel(const float *xsq, const float *xscale, int64_t n, int64_t ngroups,
                                  float4 *out) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  float mq = __int_as_float(0x7f800000), mn = __int_as_float(0x7f800000), mx = 0.0f;
  for (int64_t r = 32 * g; r < n && r < 32 * g + 32; ++r) {
    mq = fminf(mq, xsq[r]);
    mn = fminf(mn, xscale[r]);
    mx = fmaxf(mx, xscale[r]);
  }
  out[g] = make_float4(mq, mn, mx, 0.0f);
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

// Shared memory of the scan kernel: alignment slack, the query tile (and
// the fold's A block), the ring, barriers and the hit staging.
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

// The pivot pass of the probed schedule: BF16 over the pivots' image, in
// the index's metric, each query's nearest pivot (argmin mode).
static int launch_pivot_pass(int metric, const CUtensorMap &ta, const LpParams &p, cudaStream_t s) {
  switch (metric) {
    case M_L2: return launch_lp3<HORA_PREC_BF16, M_L2, TILE_ARGMIN>(ta, p, s);
    case M_IP: return launch_lp3<HORA_PREC_BF16, M_IP, TILE_ARGMIN>(ta, p, s);
    case M_COS: return launch_lp3<HORA_PREC_BF16, M_COS, TILE_ARGMIN>(ta, p, s);
  }
  return fail(HORA_EMETRIC, "no tensor-core form for this metric");
}

// The probe's keys: the scan kernel over the members' image in TILE_DIST
// mode, one CTA per work item (the grid an upper bound on their number).
template <int PREC, int MT>
static int launch_probe_items3(const CUtensorMap &ta, const LpParams &p, int max_items, cudaStream_t s) {
  const int smem = lp_smem_bytes(p.nkb, p.stages, PREC == HORA_PREC_BF16 && MT == M_L2);
  HORA_SMEM_ATTR((lowp_tile_kernel<PREC, MT, TILE_DIST>), smem);
  if (max_items <= 0) return HORA_OK;
  lowp_tile_kernel<PREC, MT, TILE_DIST><<<(unsigned)max_items, kLpThreads, smem, s>>>(ta, p);
  HORA_LAUNCHED();
  return HORA_OK;
}

static int launch_probe_items(int prec, int metric, const CUtensorMap &ta, const LpParams &p, int max_items,
                              cudaStream_t s) {
  const bool bf = prec == HORA_PREC_BF16;
  switch (metric) {
    case M_L2: return bf ? launch_probe_items3<HORA_PREC_BF16, M_L2>(ta, p, max_items, s)
                         : launch_probe_items3<HORA_PREC_FP8, M_L2>(ta, p, max_items, s);
    case M_IP: return bf ? launch_probe_items3<HORA_PREC_BF16, M_IP>(ta, p, max_items, s)
                         : launch_probe_items3<HORA_PREC_FP8, M_IP>(ta, p, max_items, s);
    case M_COS: return bf ? launch_probe_items3<HORA_PREC_BF16, M_COS>(ta, p, max_items, s)
                          : launch_probe_items3<HORA_PREC_FP8, M_COS>(ta, p, max_items, s);
  }
  return fail(HORA_EMETRIC, "no tensor-core form for this metric");
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
      }
      if (h->metric != M_COS) {
        // raw BF16 rows: the largest rounding residual (certified bounds)
        HORA_LAUNCHED();
        HORA_TRY(st->dxmax.reserve(sizeof(float)));
        HORA_CUDA_TRY(cudaMemsetAsync(st->dxmax.ptr, 0, sizeof(float), s));
        if (h->metric == M_L2) HORA_TRY(st->dxrow.reserve(sizeof(float) * std::max<int64_t>(h->n, 1)));
        bf16_residual_max_kernel<<<ceil_div(h->n, 8), 256, 0, s>>>(
            h->base.as<float>(), h->n, h->ld, h->dim, st->dxmax.as<unsigned>(),
            h->metric == M_L2 ? st->dxrow.as<float>() : nullptr);
      }
    } else {
      HORA_TRY(st->xscale.reserve(sizeof(float) * std::max<int64_t>(h->n, 1)));
      to_e4m3_kernel<<<ceil_div(h->n, 8), 256, 0, s>>>(h->base.as<float>(), h->n, h->ld, h->dim, Dp,
                                                       rows.as<uint8_t>(), st->xscale.as<float>());
    }
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<ceil_div(h->n, 256), 256, 0, s>>>(h->xsq64.as<double>(), h->n, st->xsq.as<float>());
    HORA_LAUNCHED();
    if (prec == HORA_PREC_FP8) {
      const int64_t ng = ntiles * (kLpBN / 32);  // every group of the image's tiles
      HORA_TRY(st->gmeta.reserve(sizeof(float4) * ng));
      group_meta_kernel<<<(unsigned)ceil_div(ng, (int64_t)256), 256, 0, s>>>(st->xsq.as<float>(), st->xscale.as<float>(),
                                                                             h->n, ng, st->gmeta.as<float4>());
      HORA_LAUNCHED();
    }
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
  return h->bf_probe && (h->precision == HORA_PREC_BF16 || h->precision == HORA_PREC_FP8) &&
         (h->metric == M_L2 || h->metric == M_IP || h->metric == M_COS) && h->n >= kProbeMinRows;
}

// A row image (see RowImage) of nimg rows (a multiple of the tile): image
// row i holds base row rowmap[i] (device array; 0xffffffff: padding).
static int build_row_image(hora_index *h, const LowpState &L, const uint32_t *rowmap, int64_t nimg, RowImage &out,
                           cudaStream_t s) {
  const int prec = L.prec;
  const int64_t ld = h->ld, Dp = L.Dp;
  const int nkb = (int)(Dp / (prec == HORA_PREC_BF16 ? 64 : 128));
  const int64_t esz = prec == HORA_PREC_BF16 ? 2 : 1;
  const bool fold = prec == HORA_PREC_BF16 && h->metric == M_L2, cos = h->metric == M_COS;
  const int64_t ntiles = nimg / kLpBN;
  DevBuf rowsf, sq64, rows, normblk;  // staging, freed on return
  HORA_TRY(rowsf.reserve(sizeof(float) * nimg * ld));
  HORA_TRY(sq64.reserve(sizeof(double) * nimg));
  HORA_TRY(rows.reserve(nimg * Dp * esz));
  HORA_TRY(out.xsq.reserve(sizeof(float) * nimg));
  if (prec == HORA_PREC_FP8) HORA_TRY(out.xscale.reserve(sizeof(float) * nimg));
  if (cos) HORA_TRY(out.xnorm.reserve(sizeof(float) * nimg));
  if (fold) HORA_TRY(normblk.reserve(nimg * 16 * 2));
  HORA_TRY(out.tiles.reserve(ntiles * L.tile_bytes));
  gather_members_kernel<<<(unsigned)ceil_div(nimg * ld, 256), 256, 0, s>>>(
      h->base.as<float>(), ld, rowmap, nimg, h->xsq64.as<double>(), L.xsq.as<float>(),
      cos ? h->xnorm.as<float>() : nullptr, rowsf.as<float>(), sq64.as<double>(), out.xsq.as<float>(),
      cos ? out.xnorm.as<float>() : nullptr);
  HORA_LAUNCHED();
  if (prec == HORA_PREC_BF16) {
    to_bf16_kernel<<<(unsigned)ceil_div(nimg * Dp, 256), 256, 0, s>>>(rowsf.as<float>(), nimg, ld, h->dim, Dp,
                                                                      cos ? sq64.as<double>() : nullptr,
                                                                      rows.as<__nv_bfloat16>());
    HORA_LAUNCHED();
    if (fold) {
      norm_block_kernel<<<(unsigned)ceil_div(nimg, 256), 256, 0, s>>>(sq64.as<double>(), nimg,
                                                                       normblk.as<__nv_bfloat16>());
      HORA_LAUNCHED();
    }
  } else {
    to_e4m3_kernel<<<(unsigned)ceil_div(nimg, 8), 256, 0, s>>>(rowsf.as<float>(), nimg, ld, h->dim, Dp,
                                                               rows.as<uint8_t>(), out.xscale.as<float>());
    HORA_LAUNCHED();
    HORA_TRY(out.gmeta.reserve(sizeof(float4) * (nimg / 32)));
    group_meta_kernel<<<(unsigned)ceil_div(nimg / 32, (int64_t)256), 256, 0, s>>>(
        out.xsq.as<float>(), out.xscale.as<float>(), nimg, nimg / 32, out.gmeta.as<float4>());
    HORA_LAUNCHED();
  }
  const int64_t chunks = ntiles * kLpBN * (nkb * 8 + (fold ? 2 : 0));
  tile_image_kernel<<<(unsigned)ceil_div(chunks, 256), 256, 0, s>>>(rows.as<uint8_t>(), nimg, Dp * esz, nkb,
                                                                    fold ? normblk.as<uint8_t>() : nullptr,
                                                                    L.tile_bytes, ntiles, out.tiles.as<uint8_t>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  out.rows = nimg;
  return HORA_OK;
}

// The members' image of the L.pc pivot clusters (member offsets off, C + 1
// of them) and the sample image (see LowpState).
static int build_probe_images(hora_index *h, LowpState &L, const std::vector<int64_t> &off, cudaStream_t s) {
  const int C = L.pc;
  std::vector<int64_t> moff(C + 1, 0);
  for (int c = 0; c < C; ++c)
    moff[c + 1] = moff[c] + round_up(std::min<int64_t>(off[c + 1] - off[c], kProbeMaxMembers), kLpBN);
  const int64_t nimg = moff[C];
  const int64_t ns = round_up(std::min<int64_t>(h->n, kProbeSampleRows), kLpBN);
  DevBuf rowmap;
  HORA_TRY(rowmap.reserve(sizeof(uint32_t) * std::max(nimg, ns)));
  HORA_TRY(L.moff.reserve(sizeof(int64_t) * (C + 1)));
  HORA_CUDA_TRY(cudaMemcpyAsync(L.moff.ptr, moff.data(), sizeof(int64_t) * (C + 1), cudaMemcpyHostToDevice, s));
  member_rows_kernel<<<(unsigned)ceil_div(nimg, 256), 256, 0, s>>>(L.coff.as<int64_t>(), L.cmem.as<uint32_t>(),
                                                                   L.moff.as<int64_t>(), C, nimg,
                                                                   rowmap.as<uint32_t>());
  HORA_LAUNCHED();
  HORA_TRY(build_row_image(h, L, rowmap.as<uint32_t>(), nimg, L.members, s));
  sample_rows_kernel<<<(unsigned)ceil_div(ns, 256), 256, 0, s>>>(h->n, std::min<int64_t>(h->n, kProbeSampleRows), ns,
                                                                 rowmap.as<uint32_t>());
  HORA_LAUNCHED();
  return build_row_image(h, L, rowmap.as<uint32_t>(), ns, L.sample, s);
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
  // pivots left without members (the dissolved ones, and any that lost
  // every row in the last assignment) are dropped, so that no metric's pivot
  // pass can pick an empty cluster: the member ranges stay as they are
  int Cn = 0;
  std::vector<int64_t> off;  // the kept clusters' member offsets
  {
    std::vector<float> hc((size_t)C * ld);
    HORA_CUDA_TRY(cudaMemcpyAsync(h_cnt.data(), cnt.ptr, sizeof(int64_t) * C, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(h_off.data(), L.coff.ptr, sizeof(int64_t) * (C + 1), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(hc.data(), L.centers.ptr, sizeof(float) * C * ld, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    for (int c = 0; c < C; ++c) {
      if (h_cnt[c] == 0) continue;
      if (Cn != c) std::copy(hc.begin() + (size_t)c * ld, hc.begin() + (size_t)(c + 1) * ld, hc.begin() + (size_t)Cn * ld);
      off.push_back(h_off[c]);
      ++Cn;
    }
    off.push_back(h_off[C]);
    HORA_CUDA_TRY(cudaMemcpyAsync(L.centers.ptr, hc.data(), sizeof(float) * Cn * ld, cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaMemcpyAsync(L.coff.ptr, off.data(), sizeof(int64_t) * (Cn + 1), cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the host copies are freed on return
  }
  HORA_CUDA_TRY(cudaMemsetAsync(L.xsqmax.ptr, 0, sizeof(float), s));
  max_nonneg_kernel<<<152, 256, 0, s>>>(L.xsq.as<float>(), n, L.xsqmax.as<unsigned>());
  HORA_LAUNCHED();
  // the pivots' tile image in BF16 whatever the base's precision, laid out
  // like a BF16 base of the index's metric: folded norms for Euclidean,
  // unit rows for CosineSimilarity
  const bool fold = h->metric == M_L2;
  const int64_t Dp = round_up((int64_t)h->dim, 64);
  const int nkb = (int)(Dp / 64);
  L.cnkb = nkb;
  L.ctile_bytes = (int64_t)nkb * kLpBN * 128 + (fold ? kNormBytesB : 0);
  const int64_t ctiles = ceil_div((int64_t)Cn, (int64_t)kLpBN);
  DevBuf crow, cnorm, csq;
  HORA_TRY(crow.reserve(sizeof(__nv_bfloat16) * Cn * Dp));
  HORA_TRY(cnorm.reserve(sizeof(__nv_bfloat16) * Cn * 16));
  HORA_TRY(csq.reserve(sizeof(double) * Cn));
  HORA_TRY(L.ctiles.reserve(ctiles * L.ctile_bytes));
  HORA_TRY(launch_row_norms(L.centers.as<float>(), Cn, ld, h->dim, nullptr, csq.as<double>(), s));
  to_bf16_kernel<<<ceil_div((int64_t)Cn * Dp, 256), 256, 0, s>>>(L.centers.as<float>(), Cn, ld, h->dim, Dp,
                                                                 h->metric == M_COS ? csq.as<double>() : nullptr,
                                                                 crow.as<__nv_bfloat16>());
  HORA_LAUNCHED();
  if (fold) {
    norm_block_kernel<<<ceil_div((int64_t)Cn, 256), 256, 0, s>>>(csq.as<double>(), Cn, cnorm.as<__nv_bfloat16>());
    HORA_LAUNCHED();
  }
  tile_image_kernel<<<ceil_div(ctiles * kLpBN * (nkb * 8 + 2), 256), 256, 0, s>>>(
      crow.as<uint8_t>(), Cn, Dp * 2, nkb, fold ? cnorm.as<uint8_t>() : nullptr, L.ctile_bytes, ctiles,
      L.ctiles.as<uint8_t>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the temporaries are freed on return
  L.pc = Cn;
  return build_probe_images(h, L, off, s);
}

// The sampled threshold of a wide R-best list (see the note on starting
// thresholds) into ws.ptau.  The first ms rows of the sample image are an
// even sample of the base: where r = R ms / n of them are expected below
// the base's R-th key, the rs-th smallest sample key, rs = r + 4 sqrt(r) + 2,
// has about R rs / r base rows below it, and at least R unless the sample
// count strays 4 standard deviations.  The sample is scanned by the scan kernel in two chunks with
// the search's own queries: the first s1 = 2,048 rows densely (their rs
// smallest keys, sorted), then the rest in filter mode from the k1-th of
// those keys (the same rule with r1 = R s1 / n: a loose threshold, often
// already well below the members' bound), merged into the same list; the
// threshold is its rs-th key (or the k1-th when the list stays shorter).
// Not a bound: a query that keeps fewer than R rows is answered by the
// chunked schedule.  *used is false when the sample would hold fewer than 16
// expected rows below the R-th key (a quarter of the base at most).
static int sample_threshold(hora_index *h, LowpState &L, int prec, int64_t nq, int R, SearchWorkspace &ws,
                            const CUtensorMap &ta, const LpParams &lp, cudaStream_t s, bool *used) {
  *used = false;
  const int64_t n = h->n;
  const int64_t lim = std::min<int64_t>(std::min<int64_t>(n, kProbeSampleRows), n / 4) / kLpBN * kLpBN;
  const int64_t ms = std::min<int64_t>(lim, round_up(ceil_div((int64_t)64 * n, (int64_t)R), kLpBN));
  const double r = (double)R * (double)ms / (double)n;
  if (r < 16.0) return HORA_OK;
  const int rs = (int)std::ceil(r + 4.0 * std::sqrt(r)) + 2;
  const int64_t s1 = std::min<int64_t>(ms, 2048);
  const double r1 = (double)R * (double)s1 / (double)n;
  const int k1 = std::min(rs, (int)std::ceil(r1 + 4.0 * std::sqrt(r1)) + 2);
  const int caps = (int)round_up(std::max<int64_t>(s1, 4 * rs), 128);
  int64_t nres = 1024;
  while (nres < nq) nres <<= 1;
  HORA_TRY(ws.ptau.reserve(sizeof(float) * nres));
  const int64_t lb = round_up(nq * rs, 32);  // the candidates start 256-byte aligned
  HORA_TRY(ws.sbuf.reserve(sizeof(uint64_t) * (lb + nq * caps) + sizeof(uint32_t) * nq + nq + 64));
  uint64_t *sbest = ws.sbuf.as<uint64_t>(), *scand = sbest + lb;
  uint32_t *scount = reinterpret_cast<uint32_t *>(scand + nq * caps), *sovc = scount + nq;
  uint8_t *sflags = reinterpret_cast<uint8_t *>(sovc + 4);
  float *tau = ws.ptau.as<float>();
  HORA_CUDA_TRY(cudaMemsetAsync(sbest, 0xff, sizeof(uint64_t) * nq * rs, s));
  HORA_CUDA_TRY(cudaMemsetAsync(scount, 0, sizeof(uint32_t) * (nq + 4) + nq, s));
  LpParams u = lp;
  u.tiles = L.sample.tiles.as<uint8_t>();
  u.xsq = L.sample.xsq.as<float>();
  u.xscale = L.sample.xscale.as<float>();
  u.xnorm = L.sample.xnorm.as<float>();
  u.gmeta = L.sample.gmeta.as<float4>();
  u.nq = nq;
  u.qmap = nullptr;
  u.dense_hits = 0;
  u.best = sbest;
  u.k = rs;
  u.cand = scand;
  u.cap = caps;
  u.count = scount;
  u.items = nullptr;
  auto scan = [&](int mode) -> int {
    ProfScope ps("probe_sample", s);
    return prec == HORA_PREC_BF16 ? launch_lp2<HORA_PREC_BF16>(h->metric, mode, ta, u, s)
                                  : launch_lp2<HORA_PREC_FP8>(h->metric, mode, ta, u, s);
  };
  u.r_begin = 0;
  u.r_end = s1;
  u.tpc = lp_tiles_per_cta(nq, s1);
  u.tau0 = nullptr;
  HORA_TRY(scan(TILE_DENSE));
  HORA_TRY(launch_merge_topk(sbest, rs, scand, nullptr, caps, (int)s1, nullptr, nq, sflags, sovc, s, true));
  sample_tau_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(sbest, rs, k1, nq, true, tau);
  HORA_LAUNCHED();
  if (ms > s1) {
    u.r_begin = s1;
    u.r_end = ms;
    u.tpc = lp_tiles_per_cta(nq, ms - s1);
    u.tau0 = tau;
    HORA_TRY(scan(TILE_FILTER));
    HORA_TRY(launch_merge_topk(sbest, rs, scand, scount, caps, 0, nullptr, nq, sflags, sovc, s, false));
    sample_tau_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(sbest, rs, rs, nq, false, tau);
    HORA_LAUNCHED();
  }
  *used = true;
  return HORA_OK;
}

// Starting thresholds of nq staged queries (ws.q f32, ws.lq, ws.lqsq) into
// ws.ptau, for R-best lists up to kProbeClusterMaxR wide.  lp carries the
// search's scan parameters; the pivot pass keeps each query's nearest pivot
// key in ws.pkeys.  ta16: the queries' BF16 tile map for the pivot pass (it
// runs in BF16 whatever the base's precision, in the index's metric: unit
// queries for CosineSimilarity); the probe scores members in the base's
// precision (prec) and metric, from ws.lq (and ws.lqscale for FP8).
// *order (when given) receives the queries in order of their nearest pivot
// (ws.pmem), *tq the tile map of their rows gathered in that order (ws.pqg,
// valid until the next search on this workspace).
static int probe_thresholds(hora_index *h, LowpState &L, int prec, int64_t nq, int R, int64_t Dp,
                            SearchWorkspace &ws, const CUtensorMap &ta16, const LpParams &lp, cudaStream_t s,
                            const float *slack = nullptr, const uint32_t **order = nullptr,
                            CUtensorMap *tq_out = nullptr) {
  const int C = L.pc;
  // sized for a power of two of at least 1,024 queries: a serving slot whose
  // batches vary reallocates (and with that waits for the device) rarely
  int64_t nres = 1024;
  while (nres < nq) nres <<= 1;
  HORA_TRY(ws.pkeys.reserve(sizeof(uint64_t) * nres));
  HORA_TRY(ws.poff.reserve(sizeof(int64_t) * (C + 1)));
  HORA_TRY(ws.pmem.reserve(sizeof(uint32_t) * nres));
  HORA_TRY(ws.pdist.reserve(sizeof(float) * nres * kProbeMaxMembers));
  HORA_TRY(ws.ptau.reserve(sizeof(float) * nres + sizeof(uint32_t) * nres));  // thresholds, then positions
  int64_t *qoff = ws.poff.as<int64_t>();
  uint32_t *pmem = ws.pmem.as<uint32_t>(), *pos_of = ws.ptau.as<uint32_t>() + nres;
  // nearest pivot: the tensor-core scan over the pivots' image, each drain
  // thread's smallest key combined by a 64-bit atomic minimum per query (no
  // per-pivot keys written)
  LpParams a = lp;
  a.tiles = L.ctiles.as<uint8_t>();
  a.r_begin = 0;
  a.r_end = C;
  a.tpc = lp_tiles_per_cta(nq, C);
  a.tau0 = nullptr;
  a.dense_hits = 0;
  a.nkb = L.cnkb;
  a.stages = lp_stages(L.cnkb, h->metric == M_L2);
  uint64_t *pk = ws.pkeys.as<uint64_t>();
  a.best = pk;
  HORA_CUDA_TRY(cudaMemsetAsync(pk, 0xff, sizeof(uint64_t) * nq, s));
  HORA_TRY(launch_pivot_pass(h->metric, ta16, a, s));
  fill_empty_pivot_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(pk, nq, C);
  HORA_LAUNCHED();
  // queries bucketed by pivot: position i of the pivot order holds query pmem[i]
  HORA_TRY(sort_labels(pk, nullptr, nq, C, ws.pblk, ws.pcnt, qoff, pmem, s));
  if (order) *order = pmem;
  const int mt = h->metric;
  {
    // the queries gathered in pivot order, one work item per (pivot, up to
    // 128 of its queries), the members' keys by the scan kernel
    ProfScope ps("probe_scores", s);
    const int64_t esz = prec == HORA_PREC_BF16 ? 2 : 1;
    const int64_t max_items = C + ceil_div(nq, (int64_t)kLpBM);
    const int64_t qb = round_up(nq * Dp * esz, 16);
    HORA_TRY(ws.pqg.reserve(qb + sizeof(int4) * max_items + 16));
    int4 *items = reinterpret_cast<int4 *>(ws.pqg.as<uint8_t>() + qb);
    int *n_items = reinterpret_cast<int *>(items + max_items);
    inverse_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(pmem, nq, pos_of);
    HORA_LAUNCHED();
    gather_rows_u8_kernel<<<(unsigned)nq, 128, 0, s>>>(ws.lq.as<uint8_t>(), Dp * esz,
                                                        reinterpret_cast<const int *>(pmem), nq,
                                                        ws.pqg.as<uint8_t>());
    HORA_LAUNCHED();
    probe_items_kernel<<<1, 1024, 0, s>>>(qoff, L.coff.as<int64_t>(), L.moff.as<int64_t>(), C, items, n_items);
    HORA_LAUNCHED();
    CUtensorMap tq;
    HORA_TRY(make_tmap(&tq, ws.pqg.ptr, prec, Dp, nq, kLpBM));
    if (tq_out) *tq_out = tq;
    LpParams t = lp;
    t.tiles = L.members.tiles.as<uint8_t>();
    t.xsq = L.members.xsq.as<float>();
    t.xscale = L.members.xscale.as<float>();
    t.xnorm = L.members.xnorm.as<float>();
    t.nq = nq;
    t.qmap = reinterpret_cast<const int *>(pmem);
    t.tau0 = nullptr;
    t.dense_hits = 0;
    t.items = items;
    t.n_items = n_items;
    t.out_dist = ws.pdist.as<float>();
    t.ldo = kProbeMaxMembers;
    HORA_TRY(launch_probe_items(prec, mt, tq, t, (int)max_items, s));
  }
  ProfScope ps("probe_select", s);
  probe_select_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(pk, L.coff.as<int64_t>(), C, ws.pdist.as<float>(),
                                                                pos_of, ws.lqsq.as<float>(), L.xsqmax.as<float>(),
                                                                mt, nq, R, slack, ws.ptau.as<float>());
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

int lowp_probe_kind(const hora_index *h, int R) {
  const int64_t kbe = h->precision == HORA_PREC_BF16 ? 64 : 128;
  if (!probe_eligible(h) || R > kProbeMaxR || round_up((int64_t)h->dim, kbe) / kbe > 2) return 0;
  return R <= kProbeClusterMaxR ? 1 : 2;
}

int lowp_rerank_width(const hora_index *h, int k) {
  const int64_t kbe = h->precision == HORA_PREC_BF16 ? 64 : 128;
  if (h->metric == M_L1 || round_up((int64_t)h->dim, kbe) / kbe > 2) return 0;  // the exact path answers
  int R = h->rerank > 0 ? h->rerank
                        : (h->precision == HORA_PREC_BF16 ? std::max(2 * k, k + 64) : std::max(4 * k, k + 128));
  R = std::max(R, k);
  return (int)std::min<int64_t>(R, std::max<int64_t>(h->n, k));
}

__global__ void exact_tc_slack_kernel(const float *Q, int64_t nq, int64_t ld, int64_t dim, int64_t Dp,
                                      const double *qsq64, const float *dxmax, const float *xsqmax,
                                      float *slack);

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
  // the overflow rescans' merge holds the list and the candidates in shared memory
  while (cap > 2 * R && merge_smem_bytes(R, cap) > 200 * 1024) cap -= 128;
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
  p.gmeta = L.gmeta.as<float4>();
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
    HORA_TRY(launch_merge_topk(bestR, R, c.cand, count, cap, (int)c0, qlist, nl, flags, ovc, s, false, true));
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
      HORA_TRY(launch_merge_topk(bestR, R, c.cand, count, cap, 0, qlist, nl, flags, ovc, s, false, true));
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
  const uint32_t *rr_order = nullptr;  // the rerank's query order (clusters: by nearest pivot)
  bool probe = false;                  // a starting threshold per query
  CUtensorMap tf = ta;                 // the filter pass's query rows ...
  const int *fmap = nullptr;           // ... and their query ids (null: in query order)
  if (probe_eligible(h) && R > kProbeClusterMaxR && R <= kProbeMaxR) {
    HORA_TRY(ensure_pivots(h, L, s));
    HORA_TRY(sample_threshold(h, L, prec, nq, R, ws, ta, p, s, &probe));
  } else if (probe_eligible(h) && R <= kProbeClusterMaxR) {
    probe = true;
    HORA_TRY(ensure_pivots(h, L, s));
    CUtensorMap ta16 = ta;
    if (prec == HORA_PREC_FP8) {
      // the pivot pass reads the queries in BF16 (unit rows for CosineSimilarity)
      const int64_t Dp16 = round_up((int64_t)h->dim, 64);
      HORA_TRY(ws.lq16.reserve(std::max<int64_t>(nq, 1) * Dp16 * 2));
      to_bf16_kernel<<<ceil_div(nq * Dp16, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp16,
                                                               h->metric == M_COS ? qsq64 : nullptr,
                                                               ws.lq16.as<__nv_bfloat16>());
      HORA_LAUNCHED();
      HORA_TRY(make_tmap(&ta16, ws.lq16.ptr, HORA_PREC_BF16, Dp16, nq, kLpBM));
    }
    HORA_TRY(probe_thresholds(h, L, prec, nq, R, Dp, ws, ta16, p, s, nullptr, &rr_order, &tf));
    fmap = reinterpret_cast<const int *>(rr_order);
  }
  if (probe) {
    // one filter pass from the starting thresholds; after the cluster probe
    // over the queries gathered in pivot order, so that a drain warp's 32
    // query rows share their near rows (the e4m3 slice skip is a warp vote)
    LpParams f = p;
    f.qmap = fmap;
    f.tau0 = ws.ptau.as<float>();
    f.dense_hits = 0;
    for (int64_t lo = 0; lo < n; lo += max_chunk) {
      f.r_begin = lo;
      f.r_end = std::min<int64_t>(n, lo + max_chunk);
      f.tpc = lp_tiles_per_cta(nq, f.r_end - f.r_begin);
      HORA_TRY(launch_lp(prec, h->metric, TILE_FILTER, tf, L, f, s));
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
  // A wide BF16 list is reranked only where the exact k best can lie: with
  // eps(q) a certified bound on |scan key - exact distance| (Euclidean: the
  // exact search's, see exact_tc_slack_kernel; DotProduct and
  // CosineSimilarity: rerank_slack_kernel), k candidates have exact
  // distances at most T + eps (T the k-th smallest scan key of the list),
  // so a candidate whose scan key exceeds T + 2 eps is beaten by k others
  // and cannot be among the k best: the result equals the rerank of all R.
  const bool window = prec == HORA_PREC_BF16 && L.pc > 0 && R >= 512 && R >= 4 * k;
  uint64_t *wkth = nullptr;
  uint32_t *wcount = nullptr;
  if (window) {
    HORA_TRY(ws.xslack.reserve(sizeof(float) * nq));
    HORA_TRY(ws.rwin.reserve(sizeof(uint64_t) * nq * k + sizeof(uint32_t) * nq));
    wkth = ws.rwin.as<uint64_t>();
    wcount = reinterpret_cast<uint32_t *>(wkth + nq * k);
    if (h->metric == M_L2)
      exact_tc_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, qsq64,
                                                            L.dxmax.as<float>(), L.xsqmax.as<float>(),
                                                            ws.xslack.as<float>());
    else
      rerank_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, h->metric,
                                                          qsq64, L.dxmax.as<float>(), L.xsqmax.as<float>(),
                                                          ws.xslack.as<float>());
    HORA_LAUNCHED();
  }
  auto finish = [&]() -> int {
    if (window) {
      HORA_CUDA_TRY(cudaMemsetAsync(wkth, 0xff, sizeof(uint64_t) * nq * k, s));
      HORA_TRY(launch_merge_topk(wkth, k, bestR, nullptr, R, R, nullptr, nq, flags, ovc, s, false));
      rerank_window_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(bestR, R, wkth, k, ws.xslack.as<float>(), nq,
                                                                     ws.tmp.as<uint64_t>(), wcount);
      HORA_LAUNCHED();
      HORA_TRY(launch_rerank_exact(h->metric, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim,
                                   ws.qnorm.as<float>(), h->xnorm.as<float>(), ws.tmp.as<uint64_t>(), nq, R,
                                   ws.tmp.as<uint64_t>(), s, wcount, rr_order));
      HORA_CUDA_TRY(cudaMemsetAsync(d_best, 0xff, sizeof(uint64_t) * nq * k, s));
      return launch_merge_topk(d_best, k, ws.tmp.as<uint64_t>(), wcount, R, 0, nullptr, nq, flags, ovc, s);
    }
    HORA_TRY(launch_rerank_exact(h->metric, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim,
                                 ws.qnorm.as<float>(), h->xnorm.as<float>(), bestR, nq, R,
                                 ws.tmp.as<uint64_t>(), s, nullptr, rr_order));
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
  h->last_short_lists = hs[1];
  h->last_overflow_queries = h_ovc;
  std::vector<int> redo;  // queries whose R-best lists were redone
  if (hs[1] > 0) {
    // lists the probed pass left short: the chunked schedule answers them
    h->last_probe = 2;
    const int64_t nl = hs[1];
    redo.resize(nl);
    HORA_CUDA_TRY(cudaMemcpyAsync(redo.data(), ws.qlist.ptr, sizeof(int) * nl, cudaMemcpyDeviceToHost, s));
    clear_lists_kernel<<<(unsigned)ceil_div(nl * R, 256), 256, 0, s>>>(bestR, R, ws.qlist.as<int>(), nl);
    HORA_LAUNCHED();
    CUtensorMap tg;
    HORA_TRY(gather(nl, &tg));
    HORA_TRY(chunked(tg, nl, ws.qlist.as<int>()));
    HORA_TRY(status());
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
    redo.insert(redo.end(), list.begin(), list.end());
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
  }
  h->last_retries = rounds;
  if (!redo.empty()) {
    // the exact rerank and the k best again, for the redone queries only
    std::sort(redo.begin(), redo.end());
    redo.erase(std::unique(redo.begin(), redo.end()), redo.end());
    const int64_t nl = (int64_t)redo.size();
    const int *ql = ws.qlist.as<int>();
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.qlist.ptr, redo.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, s));
    HORA_TRY(launch_rerank_exact(h->metric, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim,
                                 ws.qnorm.as<float>(), h->xnorm.as<float>(), bestR, nl, R, ws.tmp.as<uint64_t>(), s,
                                 nullptr, reinterpret_cast<const uint32_t *>(ql)));
    clear_lists_kernel<<<(unsigned)ceil_div(nl * k, 256), 256, 0, s>>>(d_best, k, ql, nl);
    HORA_LAUNCHED();
    HORA_TRY(launch_merge_topk(d_best, k, ws.tmp.as<uint64_t>(), nullptr, R, R, ql, nl, flags, ovc, s));
    // the host vector is read by the copy above before it goes out of scope
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
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
// The probe (the scan kernel on the members' image: the scan's own values,
// and delta = 1e-4 (|q|^2 + max|x|^2) added regardless) puts a query's k-th smallest
// probe value t among its pivot cluster's members.  k rows then have r <= t
// + delta + eps, so the exact k-th distance is at most that, and every row
// of the exact top k has s <= t + delta + 2 eps: the filter pass from that
// threshold keeps them all.  The kept rows are rescored exactly (reference
// op order) and the k best returned.  A query whose cluster has fewer than k
// members, or whose kept rows overflow the candidate capacity, is answered
// by the CUDA-core exact scan instead; either way the result is exact.
// DotProduct and CosineSimilarity take the same steps with their own scan
// keys, the bound eps of rerank_slack_kernel (the scan key against the
// reference's f32 dot, or its -ab / (sqrt(aa) sqrt(bb))) and the probe's
// delta for the metric (probe_bound).

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

// The certified pass keeps every row whose scan value s is within 2 eps of
// the probed threshold, eps the largest over all rows (exact_tc_slack_kernel).
// With a kept row's own norm |x| and residual |x - bf16(x)| in place of the
// largest, the same terms give its own bound e_r: its exact distance lies in
// [s - e_r, s + e_r].  The k-th smallest upper end U over the kept rows
// bounds the exact k-th distance (k rows have exact distances at most U), so
// a row with s - e_r > U is not among the exact k best.  One warp per query
// keeps the others at the front of its slots, in order, and lowers its count
// before the exact rescoring; queries with k or fewer rows, or more than
// kExactTcWindowMax (their values would not fit in the warp's registers) or
// than the capacity, keep theirs.  The bound is evaluated in f32 and widened
// by a relative 2^-8, far beyond the roundings of its dozen operations.
constexpr int kExactTcWindowMax = 1024;
__global__ void exact_tc_window_kernel(const float *Q, int64_t ld, int64_t dim, int64_t Dp, const double *qsq64,
                                       const float *xsq, const float *dxrow, int64_t nq, int k, int cap,
                                       uint64_t *cand, uint32_t *count) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const int n = (int)count[q];
  if (n <= k || n > cap || n > kExactTcWindowMax) return;
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
  const float qb = (float)(sqrt(sb) * (1.0 + 0x1p-40)), dq = (float)(sqrt(sd) * (1.0 + 0x1p-40));
  const float qsq = (float)(qsq64[q] * (1.0 + 0x1p-40)), qn = (float)(sqrt(qsq64[q]) * (1.0 + 0x1p-40));
  const float cb = (float)(Dp + 16) * 0x1p-22f, ce = (float)(dim + 4) * 0x1p-23f;
  uint64_t *kq = cand + q * (int64_t)cap;
  // e_r: exact_tc_slack_kernel's eps with the row's own |x| and residual
  auto bound = [&](uint32_t r) -> float {
    const float xs = xsq[r] * (1.0f + 0x1p-22f);
    const float xn = sqrtf(xs) * (1.0f + 0x1p-22f);
    const float dx = dxrow[r];
    const float xb = xn * (1.0f + 0x1p-8f) + dx;
    const float A = qb * dx + dq * xn;
    const float B = cb * (qb * xb + 0.5f * xs);
    const float C = 0x1p-22f * (qsq + 2.0f * qb * xb + xs);
    const float E = ce * (qn + xn) * (qn + xn);
    return (2.0f * A + 2.0f * B + C + E) * (1.0f + 0x1p-8f);
  };
  // each lane's upper ends s + e_r, ordered encoding (padding: the largest)
  uint32_t u[kExactTcWindowMax / 32];
  uint32_t lo = 0xffffffffu, hi = 0u;
#pragma unroll
  for (int i = 0; i < kExactTcWindowMax / 32; ++i) {
    const int j = lane + 32 * i;
    u[i] = 0xffffffffu;
    if (j < n) {
      const uint64_t key = kq[j];
      u[i] = f2ord(key_dist(key) + bound(key_row(key)));
      lo = min(lo, u[i]);
      hi = max(hi, u[i]);
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  // the k-th smallest upper end by a bitwise descent below the bits all of
  // them share (see probe_select_kernel), rounded up below bit 8
  const int top = 31 - __clz((int)(lo ^ hi));
  uint32_t a = top < 0 ? lo : top >= 31 ? 0u : lo & ~((2u << top) - 1u);
  for (int b = top; b >= 8; --b) {
    const uint32_t tt = a | (1u << b);
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < kExactTcWindowMax / 32; ++i) cnt += u[i] < tt;
#pragma unroll
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (cnt < k) a = tt;
  }
  const float U = ord2f(a | 0xffu);
  // keep s - e_r <= U, in order, at the front (a write never passes a read:
  // the slot written is at most the slot just read)
  int m = 0;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    uint64_t key = 0;
    bool keep = false;
    if (j < n) {
      key = kq[j];
      keep = key_dist(key) - bound(key_row(key)) <= U;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (keep) kq[m + __popc(bal & ((1u << lane) - 1u))] = key;
    m += __popc(bal);
  }
  if (lane == 0) count[q] = (uint32_t)m;
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
  return h->exact_tc && h->precision == HORA_PREC_FP32 &&
         (h->metric == M_L2 || h->metric == M_IP || h->metric == M_COS) && h->n >= kProbeMinRows &&
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
  const int mt = h->metric;
  const int stages = lp_stages(nkb, mt == M_L2);
  // BF16 queries (unit rows for CosineSimilarity), their f32 squared norms
  // and the certified slack
  HORA_TRY(ws.lq.reserve(std::max<int64_t>(nq, 1) * Dp * 2));
  HORA_TRY(ws.lerr.reserve(16));
  HORA_TRY(ws.lqsq.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  HORA_TRY(ws.xslack.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  const double *qsq64 = reinterpret_cast<const double *>(ws.qnorm.as<char>() + round_up(sizeof(float) * nq, 16));
  {
    ProfScope ps("lowp_convert", s);
    to_bf16_kernel<<<ceil_div(nq * Dp, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp,
                                                          mt == M_COS ? qsq64 : nullptr,
                                                          ws.lq.as<__nv_bfloat16>());
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(qsq64, nq, ws.lqsq.as<float>());
    HORA_LAUNCHED();
    if (mt == M_L2)
      exact_tc_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, qsq64,
                                                            L.dxmax.as<float>(), L.xsqmax.as<float>(),
                                                            ws.xslack.as<float>());
    else
      rerank_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp, mt, qsq64,
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
    HORA_TRY(launch_lp(HORA_PREC_BF16, mt, TILE_FILTER, ta, L, p, s));
  }
  // the queries the pass cannot answer (read before the merge, which
  // consumes the counts), every kept row rescored exactly, then the k best
  exact_tc_fallback_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(count, nq, k, cap, lerr + 1,
                                                                     ws.xlist.as<int>());
  HORA_LAUNCHED();
  if (mt == M_L2 && L.dxrow.ptr) {
    exact_tc_window_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(
        ws.q.as<float>(), h->ld, h->dim, Dp, qsq64, L.xsq.as<float>(), L.dxrow.as<float>(), nq, k, cap, p.cand,
        count);
    HORA_LAUNCHED();
  }
  HORA_TRY(launch_rerank_exact(mt, ws.q.as<float>(), h->ld, h->base.as<float>(), h->dim, ws.qnorm.as<float>(),
                               h->xnorm.as<float>(), p.cand, nq, cap, p.cand, s, count));
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
    // their rows (pitch ld, a multiple of 4) and then their norms
    HORA_TRY(ws.xq.reserve(sizeof(float) * nl * (h->ld + 1)));
    HORA_TRY(ws.xkeys.reserve(sizeof(uint64_t) * nl * k));
    float *xq = ws.xq.as<float>(), *xqn = xq + nl * h->ld;
    gather_rows_f32_kernel<<<ceil_div(nl * (int64_t)h->ld, 256), 256, 0, s>>>(ws.q.as<float>(), h->ld,
                                                                             ws.xlist.as<int>(), nl, xq);
    HORA_LAUNCHED();
    if (mt == M_COS) {
      gather_rows_f32_kernel<<<ceil_div(nl, 256), 256, 0, s>>>(ws.qnorm.as<float>(), 1, ws.xlist.as<int>(), nl,
                                                               xqn);
      HORA_LAUNCHED();
    }
    int retries = 0;
    HORA_TRY(bf_topk_exact(base_view(h), mt, xq, mt == M_COS ? xqn : nullptr, nl, k, h->cand_cap, ws,
                           ws.xkeys.as<uint64_t>(), s, &retries));
    scatter_keys_kernel<<<ceil_div(nl * (int64_t)k, 256), 256, 0, s>>>(ws.xkeys.as<uint64_t>(), k,
                                                                      ws.xlist.as<int>(), nl, d_best);
    HORA_LAUNCHED();
    h->last_retries = retries;
  }
  return HORA_OK;
}


// ---- the IVF coarse probe, certified on the tensor cores -------------------------------
// The reference ranks every centre by its exact FP32 distance and probes the
// pmax nearest (ties to the lower centre).  Here a BF16 pass of the scan
// kernel (dense distances) over the centres' image gives each query its
// pmax-th smallest approximate key T; with eps(q) the certified bound on
// |BF16 key - exact distance| (Euclidean: exact_tc_slack_kernel's, the
// centres playing the rows; DotProduct and CosineSimilarity:
// rerank_slack_kernel's), pmax centres have exact distances at most T + eps,
// so a centre whose approximate key exceeds T + 2 eps is beaten by pmax
// others and is not probed.  The centres within T + 2 eps are rescored in
// the reference's op order (the rerank kernel) and the pmax smallest exact
// keys kept: the FP32 probe's result.
struct CoarseTc {
  int metric = 0;
  int64_t C = 0, Dp = 0;
  int nkb = 0;
  DevBuf tiles;     // the centres' BF16 tile image (the scan's layout for the metric)
  DevBuf dxmax;     // 1 f32: the largest |c - bf16(c)| (Euclidean, DotProduct)
  DevBuf xsqmax;    // 1 f32: the largest squared centre norm
};

void coarse_tc_free(CoarseTc *p) { delete p; }

// Below this many lists the FP32 pass is the cheaper (1,024 lists: 0.24 ms
// per 10k queries against 0.30 ms for the BF16 pass with its rescoring).
constexpr int64_t kCoarseTcMinLists = 2048;

bool coarse_tc_eligible(const hora_index *h) {
  return h->exact_tc && h->kind == HORA_INDEX_IVFPQ && (int64_t)h->ivf.n_kmeans_center >= kCoarseTcMinLists &&
         (h->metric == M_L2 || h->metric == M_IP || h->metric == M_COS) && round_up((int64_t)h->dim, 64) / 64 <= 2;
}

// A query's candidate centres: those whose approximate distance (row q of
// dist) is at most the pmax-th smallest approximate key plus slack[q] (and
// a relative 2^-20 against the rounding of that f32 addition), as keys at
// the front of its C slots of out, their number to count[q].  One warp per
// query.
__global__ void coarse_window_kernel(const float *dist, int64_t C, const uint64_t *kth, int pmax,
                                     const float *slack, int64_t nq, uint64_t *out, uint32_t *count) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const uint64_t tk = kth[q * pmax + (pmax - 1)];
  float w = __int_as_float(0x7f800000);
  if (tk != kEmptyKey) {
    const float t = key_dist(tk) + slack[q];
    w = t + 0x1p-20f * fabsf(t);
  }
  uint32_t n = 0;
  for (int64_t c0 = 0; c0 < C; c0 += 32) {
    const int64_t c = c0 + lane;
    const float d = c < C ? dist[q * C + c] : __int_as_float(0x7f800000);
    const bool keep = c < C && d <= w;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) out[q * C + n + __popc(m & ((1u << lane) - 1u))] = make_key(d, (uint32_t)c);
    n += __popc(m);
  }
  if (lane == 0) count[q] = n;
}

// The exact keys of a query's candidate centres (count[q] of them at the
// front of its C slots of keys, centre rows in the low words), rescored in
// the reference's op order (the exact tile kernel's dist_op sequence over
// the dimensions; the cosine from the dot and the two norms), in place.
// One warp per query, one candidate per lane at a time.
template <int MT>
__global__ void coarse_rescore_kernel(const float *Q, int64_t ld, const float *X, int64_t dim, const float *qnorm,
                                      const float *xnorm, int64_t nq, int64_t C, const uint32_t *count,
                                      uint64_t *keys) {
  const int64_t q = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const int64_t n = (int64_t)count[q] < C ? (int64_t)count[q] : C;
  constexpr int OP = MT == M_COS ? M_IP : MT;
  for (int64_t i = lane; i < n; i += 32) {
    const uint32_t row = key_row(keys[q * C + i]);
    const float *qr = Q + q * ld, *xr = X + (int64_t)row * ld;
    float s = 0.0f;
    for (int64_t d = 0; d < dim; ++d) s = dist_op<OP>(s, qr[d], xr[d]);
    if (MT == M_COS) s = cosine_from_dot(s, qnorm[q], xnorm[row]);
    keys[q * C + i] = make_key(s, row);
  }
}

// The BF16 image of C centres (pitch h->ld) for the index's metric and
// their bound inputs (see CoarseTc), into st.
static int build_centre_image(hora_index *h, const float *centers, int64_t C, CoarseTc &st, cudaStream_t s) {
  st.metric = h->metric;
  st.C = C;
  st.Dp = round_up((int64_t)h->dim, 64);
  st.nkb = (int)(st.Dp / 64);
  const bool fold = h->metric == M_L2, cos = h->metric == M_COS;
  const int64_t ld = h->ld, Dp = st.Dp, ntiles = ceil_div(C, (int64_t)kLpBN);
  const int64_t tile_bytes = (int64_t)st.nkb * kLpBN * 128 + (fold ? kNormBytesB : 0);
  DevBuf crow, cnb, csq, csqf;  // staging, freed on return
  HORA_TRY(crow.reserve(sizeof(__nv_bfloat16) * C * Dp));
  HORA_TRY(cnb.reserve(sizeof(__nv_bfloat16) * C * 16));
  HORA_TRY(csq.reserve(sizeof(double) * C));
  HORA_TRY(csqf.reserve(sizeof(float) * C));
  HORA_TRY(st.tiles.reserve(ntiles * tile_bytes));
  HORA_TRY(st.dxmax.reserve(sizeof(float)));
  HORA_TRY(st.xsqmax.reserve(sizeof(float)));
  HORA_CUDA_TRY(cudaMemsetAsync(st.dxmax.ptr, 0, sizeof(float), s));
  HORA_CUDA_TRY(cudaMemsetAsync(st.xsqmax.ptr, 0, sizeof(float), s));
  HORA_TRY(launch_row_norms(centers, C, ld, h->dim, nullptr, csq.as<double>(), s));
  to_bf16_kernel<<<(unsigned)ceil_div(C * Dp, 256), 256, 0, s>>>(centers, C, ld, h->dim, Dp,
                                                                 cos ? csq.as<double>() : nullptr,
                                                                 crow.as<__nv_bfloat16>());
  HORA_LAUNCHED();
  if (fold) {
    norm_block_kernel<<<(unsigned)ceil_div(C, 256), 256, 0, s>>>(csq.as<double>(), C, cnb.as<__nv_bfloat16>());
    HORA_LAUNCHED();
  }
  tile_image_kernel<<<(unsigned)ceil_div(ntiles * kLpBN * (st.nkb * 8 + 2), 256), 256, 0, s>>>(
      crow.as<uint8_t>(), C, Dp * 2, st.nkb, fold ? cnb.as<uint8_t>() : nullptr, tile_bytes, ntiles,
      st.tiles.as<uint8_t>());
  HORA_LAUNCHED();
  if (!cos) {
    bf16_residual_max_kernel<<<(unsigned)ceil_div(C, 8), 256, 0, s>>>(centers, C, ld, h->dim,
                                                                       st.dxmax.as<unsigned>());
    HORA_LAUNCHED();
  }
  f64_to_f32_kernel<<<(unsigned)ceil_div(C, 256), 256, 0, s>>>(csq.as<double>(), C, csqf.as<float>());
  HORA_LAUNCHED();
  max_nonneg_kernel<<<152, 256, 0, s>>>(csqf.as<float>(), C, st.xsqmax.as<unsigned>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaStreamSynchronize(s));  // the staging buffers are freed on return
  return HORA_OK;
}

static int ensure_coarse_tc(hora_index *h, const float *centers, int64_t C, cudaStream_t s) {
  if (h->coarse_tc && h->coarse_tc->C == C && h->coarse_tc->metric == h->metric) return HORA_OK;
  std::unique_ptr<CoarseTc, CoarseTcDeleter> st(new CoarseTc());
  HORA_TRY(build_centre_image(h, centers, C, *st, s));
  h->coarse_tc = std::move(st);
  return HORA_OK;
}

// The BF16 distance pass of nq staged query rows (BF16 copy lq, pitch Dp;
// f32 squared norms qsq and norms qnorm) over a centre image: dist[q * C +
// c], the scan kernel's key for the metric.
static int centre_dist_pass(hora_index *h, const CoarseTc &T, const void *lq, int64_t nq, const float *qsq,
                            const float *qnorm, int *err, float *dist, cudaStream_t s) {
  CUtensorMap ta;
  HORA_TRY(make_tmap(&ta, lq, HORA_PREC_BF16, T.Dp, nq, kLpBM));
  LpParams p{};
  p.nq = nq;
  p.nkb = T.nkb;
  p.stages = lp_stages(T.nkb, h->metric == M_L2);
  p.tiles = T.tiles.as<uint8_t>();
  p.qsq = qsq;
  p.qnorm = qnorm;
  p.err = err;
  p.r_begin = 0;
  p.r_end = T.C;
  p.tpc = lp_tiles_per_cta(nq, T.C);
  p.out_dist = dist;
  p.ldo = T.C;
  if (h->metric == M_L2) return launch_lp3<HORA_PREC_BF16, M_L2, TILE_DIST>(ta, p, s);
  if (h->metric == M_IP) return launch_lp3<HORA_PREC_BF16, M_IP, TILE_DIST>(ta, p, s);
  return launch_lp3<HORA_PREC_BF16, M_COS, TILE_DIST>(ta, p, s);
}

// 2 eps per query row of Q (pitch ld; f64 squared norms qsq64) against the
// centres of T (see rerank_slack_kernel / exact_tc_slack_kernel).
static int centre_slack(hora_index *h, const CoarseTc &T, const float *Q, int64_t nq, const double *qsq64,
                        float *slack, cudaStream_t s) {
  if (h->metric == M_L2)
    exact_tc_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(Q, nq, h->ld, h->dim, T.Dp, qsq64, T.dxmax.as<float>(),
                                                          T.xsqmax.as<float>(), slack);
  else
    rerank_slack_kernel<<<ceil_div(nq, 8), 256, 0, s>>>(Q, nq, h->ld, h->dim, T.Dp, h->metric, qsq64,
                                                        T.dxmax.as<float>(), T.xsqmax.as<float>(), slack);
  HORA_LAUNCHED();
  return HORA_OK;
}

int coarse_tc_probe(hora_index *h, const float *centers, const float *cnorm, int64_t C, int64_t nq, int pmax,
                    SearchWorkspace &ws, float *dist, uint64_t *probes, cudaStream_t s) {
  if (nq <= 0) return HORA_OK;
  HORA_TRY(ensure_coarse_tc(h, centers, C, s));
  const CoarseTc &T = *h->coarse_tc;
  const int64_t Dp = T.Dp;
  HORA_TRY(ws.lq.reserve(nq * Dp * 2));
  HORA_TRY(ws.lqsq.reserve(sizeof(float) * nq));
  HORA_TRY(ws.lerr.reserve(16));
  HORA_TRY(ws.xslack.reserve(sizeof(float) * nq));
  HORA_TRY(ws.ccand.reserve(sizeof(uint64_t) * nq * C + sizeof(uint32_t) * nq));
  HORA_TRY(ws.ovf_flag.reserve(nq));
  HORA_TRY(ws.ovf_counter.reserve(sizeof(uint32_t)));
  uint64_t *cand = ws.ccand.as<uint64_t>();
  uint32_t *count = reinterpret_cast<uint32_t *>(cand + nq * C);
  const double *qsq64 = reinterpret_cast<const double *>(ws.qnorm.as<char>() + round_up(sizeof(float) * nq, 16));
  {
    ProfScope ps("coarse_tc", s);
    to_bf16_kernel<<<(unsigned)ceil_div(nq * Dp, 256), 256, 0, s>>>(ws.q.as<float>(), nq, h->ld, h->dim, Dp,
                                                                    h->metric == M_COS ? qsq64 : nullptr,
                                                                    ws.lq.as<__nv_bfloat16>());
    HORA_LAUNCHED();
    f64_to_f32_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(qsq64, nq, ws.lqsq.as<float>());
    HORA_LAUNCHED();
    HORA_CUDA_TRY(cudaMemsetAsync(ws.lerr.ptr, 0, 16, s));
    HORA_TRY(centre_dist_pass(h, T, ws.lq.ptr, nq, ws.lqsq.as<float>(), ws.qnorm.as<float>(), ws.lerr.as<int>(),
                              dist, s));
    HORA_TRY(centre_slack(h, T, ws.q.as<float>(), nq, qsq64, ws.xslack.as<float>(), s));
  }
  HORA_TRY(launch_rows_topk(dist, nq, C, C, pmax, probes, s));
  coarse_window_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(dist, C, probes, pmax, ws.xslack.as<float>(), nq,
                                                                 cand, count);
  HORA_LAUNCHED();
  {
    const unsigned g = (unsigned)ceil_div(nq, 8);
    if (h->metric == M_L2)
      coarse_rescore_kernel<M_L2><<<g, 256, 0, s>>>(ws.q.as<float>(), h->ld, centers, h->dim, ws.qnorm.as<float>(),
                                                    cnorm, nq, C, count, cand);
    else if (h->metric == M_IP)
      coarse_rescore_kernel<M_IP><<<g, 256, 0, s>>>(ws.q.as<float>(), h->ld, centers, h->dim, ws.qnorm.as<float>(),
                                                    cnorm, nq, C, count, cand);
    else
      coarse_rescore_kernel<M_COS><<<g, 256, 0, s>>>(ws.q.as<float>(), h->ld, centers, h->dim, ws.qnorm.as<float>(),
                                                     cnorm, nq, C, count, cand);
    HORA_LAUNCHED();
  }
  HORA_CUDA_TRY(cudaMemsetAsync(probes, 0xff, sizeof(uint64_t) * nq * pmax, s));
  HORA_TRY(launch_merge_topk(probes, pmax, cand, count, (int)C, 0, nullptr, nq, ws.ovf_flag.as<uint8_t>(),
                             ws.ovf_counter.as<uint32_t>(), s, true));
  int err = 0;
  HORA_CUDA_TRY(cudaMemcpyAsync(&err, ws.lerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  if (err) return fail(HORA_ETIMEDOUT, "tensor-core coarse pass: a pipeline wait timed out");
  return HORA_OK;
}

}  // namespace hora
