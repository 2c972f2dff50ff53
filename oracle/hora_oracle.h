/*
 * hora_oracle.h — CPU restatement of hora's search path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
 * check and the CPU-baseline leg of bench.py may load it.  The product
 * (libhora_gb300.so) never links or calls it.
 *
 * Parity status (what pins this restatement):
 *   - metrics:   pinned by the reference's known-answer tests
 *                src/core/calc.rs:46-50 (dot([1,2,3],[1,2,3]) == -14) and
 *                src/core/node.rs:178-186 (Manhattan([1,1],[2,2]) == 2);
 *                the op order follows the scalar branches of
 *                src/core/simd_metrics.rs:30-33,60-66,96-102.
 *   - brute force, k-means, PQ / IVF-PQ: restated line by line from
 *                src/index/bruteforce_idx.rs, src/core/kmeans.rs and
 *                src/index/pq_idx.rs.  The reference is Rust and no Rust
 *                toolchain exists here, so beyond the two known-answer tests
 *                these parts are "parity unpinned" against reference
 *                outputs; they are pinned by hand-derived fixtures and by
 *                the FP64 exact oracle.
 *   - CosineSimilarity: the reference computes sqrt of a negative number and
 *                yields NaN for every input (src/core/metrics.rs:79-82);
 *                the restatement implements the evident intent
 *                -dot(a,b)/(|a||b|), "smaller means closer".  Unpinned.
 *   - k-means randomness: the reference draws from an unseeded thread RNG
 *                (src/core/kmeans.rs:168); the restatement uses a seeded
 *                splitmix64 stream per k-means instance, shared bit-for-bit
 *                with the GPU build.
 */
#ifndef HORA_ORACLE_H
#define HORA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same variant order as the reference Metric enum (src/core/metrics.rs:5-13). */
enum {
  HORO_UNKNOWN = 0,
  HORO_MANHATTAN = 1,
  HORO_DOT = 2,
  HORO_EUCLIDEAN = 3,
  HORO_COSINE = 4,
  HORO_ANGULAR = 5
};

/* calc::dot — returns the NEGATED inner product (src/core/calc.rs:13-18). */
float horo_calc_dot_f32(const float *a, const float *b, int64_t d);
double horo_calc_dot_f64(const double *a, const double *b, int64_t d);

/* metrics::metric (src/core/metrics.rs:22-34).  *err = 1 for Unknown/Angular. */
float horo_metric_f32(const float *a, const float *b, int64_t d, int metric, int *err);
double horo_metric_f64(const double *a, const double *b, int64_t d, int metric, int *err);

/* BruteForceIndex::node_search_k (src/index/bruteforce_idx.rs:47-73) with the
 * std BinaryHeap eviction order.  Results nq x k ascending; slots beyond
 * min(k, n) hold idx -1 and +inf.  threads > 1 splits the queries. */
int horo_bf_search(const float *base, int64_t n, int64_t dim, const float *queries, int64_t nq,
                   int64_t k, int metric, int64_t *idx_out, float *dist_out, int threads);

/* Exact top-k with distances accumulated in double from the f32 inputs, ties
 * broken by lower index.  The recall / distance-error ground truth. */
int horo_bf_exact_f64(const float *base, int64_t n, int64_t dim, const float *queries,
                      int64_t nq, int64_t k, int metric, int64_t *idx_out, double *dist_out,
                      int threads);

/* splitmix64 stream shared with the GPU build. */
uint64_t horo_rng_instance_seed(uint64_t seed, uint64_t instance);
uint64_t horo_rng_next(uint64_t *state);
double horo_rng_unit(uint64_t *state);

/* Kmeans pieces (src/core/kmeans.rs).  Data rows have `stride` floats; the
 * k-means works on columns [begin, end) minus residual[begin..end) when
 * residual != NULL.  accum_f64 selects double accumulation of the centroid
 * sums (the GPU build's documented choice); 0 follows the reference's f32. */
void horo_kmeans_init(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                      const float *residual, int64_t n_center, int accum_f64, float *centers);
void horo_kmeans_assign(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                        const float *residual, const float *centers, int64_t n_center, int metric,
                        int64_t *assign_out);
void horo_kmeans_update(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                        const float *residual, const int64_t *assign, int64_t n_center,
                        int accum_f64, float *centers, int64_t *counts_out);
int horo_kmeans_split(float *centers, int64_t *counts, int64_t n_center, int64_t dim,
                      int64_t batch_size, uint64_t *rng_state);
int horo_kmeans_train(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                      const float *residual, int64_t n_center, int64_t n_epoch, int metric,
                      uint64_t rng_seed, int accum_f64, float *centers_out);

/* PQIndex::new subspace ranges (src/index/pq_idx.rs:75-88). */
void horo_pq_ranges(int64_t dim, int64_t n_sub, int64_t *begin_out, int64_t *end_out);

/* IVFPQIndex::train (src/index/pq_idx.rs:357-396).  Codebooks are laid out
 * [n_list][n_sub][2^sub_bits][dmax]; codes [n][n_sub] in list order (the
 * order of list_items).  train_size = 0 trains on every item (reference
 * behaviour); list_trained[c] = 0 marks an empty list (the reference panics). */
int horo_ivfpq_build(const float *data, int64_t n, int64_t dim, int64_t n_sub, int64_t sub_bits,
                     int64_t n_list, int64_t n_epoch, int metric, uint64_t seed, int accum_f64,
                     int64_t train_size, float *centers_out, int64_t *list_offsets_out,
                     int64_t *list_items_out, float *codebooks_out, uint8_t *codes_out,
                     uint8_t *list_trained_out);

/* PQ codes of `n` rows against one list's codebook (pq_idx.rs:143-144). */
void horo_pq_encode(const float *data, int64_t n, int64_t dim, const float *list_center,
                    const float *codebook, int64_t n_sub, int64_t sub_bits, uint8_t *codes_out);

/* Per-query LUT (pq_idx.rs:170-179): n_sub x 2^sub_bits floats. */
void horo_pq_lut(const float *query, int64_t dim, const float *list_center, const float *codebook,
                 int64_t n_sub, int64_t sub_bits, float *lut_out);

/* IVFPQIndex::search_knn_adc + node_search_k (pq_idx.rs:408-477). */
int horo_ivfpq_search(const float *centers, int64_t n_list, int64_t dim,
                      const int64_t *list_offsets, const int64_t *list_items,
                      const float *codebooks, const uint8_t *codes, const uint8_t *list_trained,
                      int64_t n_sub, int64_t sub_bits, int metric, const float *queries,
                      int64_t nq, int64_t k, int64_t nprobe, int64_t *idx_out, float *dist_out,
                      int threads);

/* Coarse distances of a query to every list centre (pq_idx.rs:416-421). */
void horo_ivf_coarse(const float *centers, int64_t n_list, int64_t dim, int metric,
                     const float *query, float *dist_out);

/* MLP 40->H1->H2->1 with ReLU, parameters packed as
 * [W1(H1xF) b1(H1) W2(H2xH1) b2(H2) W3(H2) b3(1)].  Forward in double. */
void horo_mlp_forward(const float *params, int64_t f, int64_t h1, int64_t h2, const float *x,
                      int64_t n, float *out);
/* Asymmetric squared error: weight `alpha` where pred < y, 1 elsewhere,
 * averaged over n.  Returns the loss, writes d loss / d params. */
double horo_mlp_loss_grad(const float *params, int64_t f, int64_t h1, int64_t h2, const float *x,
                          const float *y, int64_t n, float alpha, double *grad_out);


/* Flat PQIndex (src/index/pq_idx.rs:21-265): codebooks [n_sub][K][dmax],
 * codes [n][n_sub]; the build metric drives the k-means and the LUT. */
int horo_pq_build(const float *data, int64_t n, int64_t dim, int64_t n_sub, int64_t sub_bits,
                  int64_t n_epoch, int metric, uint64_t seed, int accum_f64, int64_t train_size,
                  float *codebooks_out, uint8_t *codes_out);
int horo_pq_search(const float *codebooks, const uint8_t *codes, int64_t n, int64_t dim,
                   int64_t n_sub, int64_t sub_bits, int metric, const float *queries, int64_t nq,
                   int64_t k, int64_t *idx_out, float *dist_out, int threads);

/* kmeans::general_kmeans (src/core/kmeans.rs:216-289).  Means start at
 * data[init_rows[i]] or, when init_rows is NULL, at k rows drawn with
 * replacement from the splitmix64 stream of `seed` (row = next * n >> 64).
 * Sums run in node order.  means_out (k x dim) receives the final means;
 * roots_out (k) per mean the nearest node.  Returns -1 for a bad init row. */
int horo_general_kmeans(const float *data, int64_t n, int64_t dim, int64_t k, int64_t epoch, int metric,
                        const int64_t *init_rows, uint64_t seed, int64_t *roots_out, float *means_out,
                        int threads);

#ifdef __cplusplus
}
#endif
#endif
