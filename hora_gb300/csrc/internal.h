// internal.h — host-side interfaces between the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace hora {

// ---- exact FP32 distance tiles (bf_fp32.cu) ----------------------------------
enum TileMode : int { TILE_FILTER = 0, TILE_DENSE = 1, TILE_ARGMIN = 2, TILE_DIST = 3 };

struct TileParams {
  const float *Q = nullptr;  // query rows (pitch ldq floats), row i read as qmap[i] if qmap
  int64_t ldq = 0;
  int64_t nq = 0;            // rows of the tile's query list
  const int *qmap = nullptr; // list slot -> query id (nullptr: identity)
  const float *X = nullptr;  // base rows (pitch ldx floats)
  int64_t ldx = 0;
  int64_t r_begin = 0, r_end = 0;  // base rows scored
  int64_t ld = 0;                  // columns scored (padded dimension)
  const float *qnorm = nullptr, *xnorm = nullptr;  // cosine only
  // TILE_FILTER / TILE_DENSE: candidate append against best[qid*k + k-1]
  uint64_t *best = nullptr;
  int k = 0;
  uint64_t *cand = nullptr;
  int cap = 0;
  uint32_t *count = nullptr;
  // TILE_ARGMIN: per query smallest (distance,row) key
  uint64_t *out_key = nullptr;
  // TILE_DIST: dense f32 distances out[qid*ldo + (row - r_begin)]
  float *out_dist = nullptr;
  int64_t ldo = 0;
};

int launch_dist_tile(int metric, int mode, const TileParams &p, cudaStream_t s);
// Copies n rows (src pitch lds, may alias dst) to dst (pitch ld, zero
// padding), raises *flag on a NaN / Inf element and writes the row norms
// (f32 and f64 squares, either may be null), in one pass.
int launch_stage_rows(const float *src, int64_t lds, int64_t n, int64_t dim, int64_t ld, float *dst,
                      uint32_t *flag, float *nf, double *sq, cudaStream_t s);
int launch_row_norms(const float *X, int64_t n, int64_t ld, int64_t dim, float *norm_f32,
                     double *sq_f64, cudaStream_t s);
int launch_check_finite(const float *X, int64_t n, int64_t ld, int64_t dim, uint32_t *flag,
                        cudaStream_t s);

// Exact FP32 distances (reference op order) for R candidate rows per query:
// in = approximate keys (row in the low word), out = exact keys.  With
// count, query q has min(count[q], R) keys in its R slots (in may be out).
// With order (a permutation of the nq queries), they are taken in that order.
int launch_rerank_exact(int metric, const float *Q, int64_t ld, const float *X, int64_t dim,
                        const float *qnorm, const float *xnorm, const uint64_t *in, int64_t nq,
                        int R, uint64_t *out, cudaStream_t s, const uint32_t *count = nullptr,
                        const uint32_t *order = nullptr);

// ---- selection (topk.cu) ------------------------------------------------------
// Merges each query's candidates into its sorted k-best key list (dedup by
// key).  dense_n > 0: candidates are the first dense_n slots, count ignored.
// sorted = false (an intermediate list) may leave the k-1 smallest keys
// unordered; the k-th (largest) key is always at position k-1.  disjoint:
// the candidates of listed queries (qlist) are rows their lists do not hold
// (a new chunk), so no deduplication is needed.
int launch_merge_topk(uint64_t *best, int k, const uint64_t *cand, uint32_t *count, int cap,
                      int dense_n, const int *qlist, int64_t nlist, uint8_t *ovf_flag,
                      uint32_t *ovf_counter, cudaStream_t s, bool sorted = true, bool disjoint = false);
int merge_smem_bytes(int k, int cap);
// Sorted keys -> (ids via the id table, distances); empty keys -> NO_ID, +inf.
int launch_keys_to_results(const uint64_t *keys, int64_t n_keys, const uint64_t *id_table,
                           uint64_t *ids_out, float *dist_out, cudaStream_t s);
// Gathers result rows for search_nodes.
int launch_gather_rows(const uint64_t *keys, int64_t n_keys, const float *base, int64_t ld,
                       int64_t dim, float *out, cudaStream_t s);
// Per-row top-k of a dense f32 matrix (rows x cols): k <= 1024.
int launch_rows_topk(const float *D, int64_t rows, int64_t cols, int64_t ldd, int k,
                     uint64_t *out_keys, cudaStream_t s);

// ---- brute force (bf_search.cu) ---------------------------------------------------
// Per-search scratch.  One workspace per concurrent search context (the
// handle owns one; every serving slot owns another), so searches on
// different contexts can run on different streams over the same index.
struct SearchWorkspace {
  DevBuf q, qnorm, best, cand, count, ovf_flag, ovf_counter, qlist, out_ids, out_dist, rows,
      keys2, tmp;
  // IVF-PQ
  DevBuf coarse, probes, pair_cnt, pair_off, pair_q, pair_c, pair_slot, ivf_cand, best_r, tmp_keys;
  DevBuf adc_next, adc_gmap;  // the ADC kernel's group counter and group -> list map
  // low-precision scoring
  DevBuf lq, lqsq, lqscale, lqgather, lerr;
  DevBuf lq16;  // an FP8 search's BF16 query copy (the pivot pass reads it)
  // BF16 starting thresholds: query -> pivot keys, queries bucketed by pivot,
  // probe distances (queries x members), thresholds
  DevBuf pkeys, poff, pmem, pblk, pcnt, pdist, ptau;
  DevBuf pqg;    // the probe's queries in pivot order and its work items
  DevBuf sbuf;   // wide lists: the sample pass's lists, candidates, counts and flags
  DevBuf rwin;   // windowed rerank: each query's k best approximate keys, then its kept counts
  DevBuf ccand;  // certified coarse probe: the centres rescored per query, then their counts
  // learned nprobe
  DevBuf feats, pred, npq;
  // certified tensor-core exact search: per-query threshold slack, one empty
  // key per query, the queries answered by the CUDA-core scan instead (list,
  // their rows, their keys)
  DevBuf xslack, xempty, xlist, xq, xkeys;
  std::vector<uint8_t> h_flags;
  // the finiteness flag of the staged queries, read before the results are written
  DevBuf d_status;
  HostBuf h_status;
  EventBox ev_status;
  bool status_pending = false;
  // device bytes the workspace holds (its buffers only grow)
  size_t device_bytes() const {
    const DevBuf *all[] = {&q, &qnorm, &best, &cand, &count, &ovf_flag, &ovf_counter, &qlist, &out_ids,
                           &out_dist, &rows, &keys2, &tmp, &coarse, &probes, &pair_cnt, &pair_off, &pair_q,
                           &pair_c, &pair_slot, &ivf_cand, &best_r, &tmp_keys, &adc_next, &adc_gmap, &lq,
                           &lqsq, &lqscale, &lqgather, &lerr, &lq16, &pkeys, &poff, &pmem, &pblk, &pcnt, &pdist,
                           &ptau, &pqg, &sbuf, &rwin, &ccand, &feats, &pred, &npq, &xslack, &xempty, &xlist, &xq, &xkeys, &d_status};
    size_t b = 0;
    for (const DevBuf *d : all) b += d->bytes;
    return b;
  }
  // the search's own start / end events (timed), created once per workspace
  EventBox ev_t0, ev_t1;
};

struct BaseView {
  const float *X;  // n x ld
  int64_t n, ld, dim;
  const float *xnorm;  // f32 norms (cosine)
};

// Exact k-best keys for nq staged queries (pitch ld) against the base.
int bf_topk_exact(const BaseView &b, int metric, const float *dQ, const float *dqnorm, int64_t nq,
                  int k, int cand_cap, SearchWorkspace &ws, uint64_t *d_best, cudaStream_t s,
                  int *retries_out);

// ---- k-means pieces (ivfpq.cu) ------------------------------------------------------
// Stable bucketing of n items by label (labels[i], or key_row(keys[i]) when
// keys is given): d_offsets (C + 1 entries) and d_members, the items of each
// bucket in item order.  counts receives the C bucket sizes.
int sort_labels(const uint64_t *keys, const uint32_t *labels, int64_t n, int C, DevBuf &blk,
                DevBuf &counts, int64_t *d_offsets, uint32_t *d_members, cudaStream_t s);
// New centres (pitch ld): per (centre, column) the sum over the bucket's
// members in item order (f32 adds, or f64 when accum_f64) divided by the
// count; an empty bucket gets `empty` in every column.
int launch_center_sum(const float *X, int64_t ld, const uint32_t *members, const int64_t *offsets,
                      int C, int64_t dim, int accum_f64, float empty, float *centers, cudaStream_t s);

// ---- error helpers ------------------------------------------------------------------
const char *metric_name(int m);

}  // namespace hora
