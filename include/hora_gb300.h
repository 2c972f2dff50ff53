/*
 * hora_gb300.h — C ABI of the GB300 implementation of hora's search path.
 *
 * One shared library, libhora_gb300.so, exports these entry points.  They
 * replace, one for one, the methods of the reference's
 *   trait ANNIndex<E, T>            src/core/ann_index.rs:25-121
 *   trait SerializableIndex<E, T>   src/core/ann_index.rs:141-158
 * as implemented by
 *   BruteForceIndex<f32, T>         src/index/bruteforce_idx.rs:15-106
 *   IVFPQIndex<f32, T> ("PQIVFIndex", README.md:57)   src/index/pq_idx.rs:267-523
 * with the element type fixed to f32 and the id type to uint64_t (a host
 * wrapper maps any other id type through a table; see hora_gb300.hpp).
 *
 * Conventions
 *  - Every call returns an int status: HORA_OK (0) or a negative HORA_E*
 *    code; hora_last_error() gives the message for the calling thread (the
 *    reference returns Result<_, &'static str> or panics; nothing panics
 *    across this ABI).
 *  - Vector arguments are row-major n x dim float32.  A pointer may be host
 *    memory or device memory of the current CUDA device; the library detects
 *    which and copies only host buffers (memory of another device is
 *    HORA_EINVAL).  The caller owns all buffers, the library owns the handle
 *    and its device memory.
 *  - Search results are nq x k, ascending distance ("smaller means closer",
 *    src/core/metrics.rs:55,78).  When fewer than k items exist the tail
 *    slots hold id HORA_NO_ID and distance +inf (the reference returns a
 *    shorter Vec).
 *  - Distances follow the reference: Euclidean is the SQUARED L2 distance
 *    (src/core/simd_metrics.rs:96-102); DotProduct is +<x,q> ascending
 *    (metrics.rs:50-57 negates calc::dot, which already negates);
 *    CosineSimilarity is -<x,q>/(|x||q|) (the reference yields NaN here,
 *    metrics.rs:79-82; this is its evident intent), 0 when a norm is 0.
 *  - Searches on one handle are serialised by the handle; add/build/clear
 *    need exclusive access, as with &mut self in the reference.
 */
#ifndef HORA_GB300_H
#define HORA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HORA_OK 0
#define HORA_EINVAL -1     /* bad argument (null pointer, k == 0 ...)       */
#define HORA_EDIM -2       /* "dimension is different" (pq_idx.rs:101-103) */
#define HORA_ECAP -3       /* size beyond a stated maximum                  */
#define HORA_EMETRIC -4    /* "unknown method" (metrics.rs:32)              */
#define HORA_ENAN -5       /* NaN / Inf element (node.rs:158-166 panics)    */
#define HORA_EOOM -6       /* device allocation failed / HBM budget         */
#define HORA_ECUDA -7      /* CUDA runtime error                            */
#define HORA_ENOTBUILT -8  /* search before build (reference panics)        */
#define HORA_ENOTIMPL -9   /* "not implement" (ann_index.rs:69-71)          */
#define HORA_EIO -10       /* dump/load file error                          */
#define HORA_ETIMEDOUT -11 /* a bounded device-side wait ran out            */
#define HORA_ESIZE -12     /* "vector's size is different with index" (:48) */

#define HORA_NO_ID UINT64_MAX

/* ---- enums --------------------------------------------------------------- */
/* Same variant order as the reference Metric enum (src/core/metrics.rs:5-13). */
typedef enum {
  HORA_METRIC_UNKNOWN = 0,
  HORA_METRIC_MANHATTAN = 1,
  HORA_METRIC_DOT_PRODUCT = 2,
  HORA_METRIC_EUCLIDEAN = 3,
  HORA_METRIC_COSINE_SIMILARITY = 4,
  HORA_METRIC_ANGULAR = 5 /* kept for the enum order; not supported */
} hora_metric;

typedef enum {
  HORA_INDEX_BRUTE_FORCE = 0, /* BruteForceIndex */
  HORA_INDEX_IVFPQ = 1,       /* IVFPQIndex */
  HORA_INDEX_PQIVF = 1,       /* README name of the same index */
  HORA_INDEX_PQ = 2           /* PQIndex (flat; src/index/pq_idx.rs:21-265) */
} hora_index_kind;

/* Scoring precision of brute-force search (GPU-only knob).  The approximate
 * forms score every row in reduced precision, keep a widened candidate list
 * and rerank it exactly in FP32, so returned distances are always the
 * exact FP32 ones. */
typedef enum {
  HORA_PREC_FP32 = 0, /* exact: reference op order, bit-identical distances */
  HORA_PREC_BF16 = 1, /* tcgen05 BF16 GEMM scoring + FP32 rerank            */
  HORA_PREC_FP8 = 2   /* tcgen05 FP8 e4m3 (per-row scale) + FP32 rerank     */
} hora_precision;

/* ---- params (src/index/pq_params.rs:43-91, bruteforce_params.rs:5-14) ---- */
typedef struct {
  uint32_t reserved; /* BruteForceParams {} has no fields */
} hora_bf_params;

typedef struct {
  uint64_t n_sub;           /* default 25  */
  uint64_t sub_bits;        /* default 4   (1..8 supported: u8 codes) */
  uint64_t n_kmeans_center; /* default 256 */
  uint64_t search_n_center; /* default 8   (nprobe) */
  uint64_t train_epoch;     /* default 100 */
} hora_ivfpq_params;

/* PQParams (src/index/pq_params.rs:8-41). */
typedef struct {
  uint64_t n_sub;       /* default 4   */
  uint64_t sub_bits;    /* default 4   (1..8 supported: u8 codes) */
  uint64_t train_epoch; /* default 100 */
} hora_pq_params;

/* GPU-only options, set per handle with hora_set_option(key, value). */
typedef enum {
  HORA_OPT_PRECISION = 1,      /* hora_precision for brute force, default FP32 */
  HORA_OPT_RERANK = 2,         /* candidates kept for the FP32 rerank (0 = auto) */
  HORA_OPT_SEED = 3,           /* k-means RNG seed, default 0x686f7261 */
  HORA_OPT_TRAIN_SIZE = 4,     /* IVF-PQ: train on the first N items (0 = all) */
  HORA_OPT_ACCUM_F64 = 5,      /* k-means centroid sums in FP64 (default 1) */
  HORA_OPT_CAND_CAP = 6,       /* brute-force per-query candidate capacity */
  HORA_OPT_LEARNED_NPROBE = 7, /* IVF-PQ: use the trained nprobe model (0/1) */
  HORA_OPT_NPROBE_MARGIN = 8,  /* learned nprobe: margin in log2 units added to
                                  the one training calibrated (default 0) */
  HORA_OPT_NPROBE_MAX = 9,     /* learned nprobe: upper clamp */
  HORA_OPT_IVF_RERANK = 10,    /* IVF-PQ: exact FP32 rerank of this many ADC
                                  candidates (0 = off, reference behaviour) */
  HORA_OPT_NPROBE_PHASE1 = 11, /* learned nprobe: lists probed before the model
                                  reads its features (0..64, default 4; fixed at
                                  training) */
  HORA_OPT_BF_PROBE = 12,      /* BF16 / FP8 brute force (Euclidean, DotProduct,
                                  CosineSimilarity) on >= 65,536 rows: start each
                                  query's scan from a threshold, probed in its
                                  nearest pivot cluster (R-best lists up to 256)
                                  or taken from an even sample of the base (wider
                                  lists, up to 4,096), then one pass over the base
                                  (default 1; 0 = chunked schedule only; same
                                  results either way) */
  HORA_OPT_EXACT_TC = 13       /* exact FP32 brute force (Euclidean, DotProduct,
                                  CosineSimilarity) on >= 65,536 rows, dim <=
                                  128, k <= 256: the BF16 tensor-core scan as a
                                  filter certified by a rounding-error bound, then
                                  every kept row rescored exactly; and the coarse
                                  probe of an IVF-PQ index of >= 2,048 lists: a
                                  BF16 pass, then the centres within the bound of
                                  the nprobe-th rescored exactly (default 1; 0 =
                                  the CUDA-core FP32 passes; same results either
                                  way) */
} hora_option;

typedef struct hora_index hora_index;

/* ---- lifecycle --------------------------------------------------------- */
/* BruteForceIndex::new (bruteforce_idx.rs:25) / IVFPQIndex::new (pq_idx.rs:295)
 * / PQIndex::new (pq_idx.rs:48-90).  params points to hora_bf_params,
 * hora_ivfpq_params or hora_pq_params (NULL = defaults).  A PQIndex trains
 * its codebooks on the raw vectors with the build metric (CosineSimilarity
 * is rejected: the reference's metric is NaN there and its heap panics). */
int hora_index_create(int kind, uint64_t dim, const void *params, hora_index **out);
int hora_index_free(hora_index *h);
void hora_ivfpq_params_default(hora_ivfpq_params *p); /* pq_params.rs:80-91 */
void hora_pq_params_default(hora_pq_params *p);       /* pq_params.rs:32-41 */

/* ---- ANNIndex ---------------------------------------------------------- */
/* add_node / add / madd (ann_index.rs:36-59): n vectors with their ids. */
int hora_add(hora_index *h, const float *vecs, const uint64_t *ids, uint64_t n);
/* build (ann_index.rs:30): BF stores the metric (bruteforce_idx.rs:36-39);
 * IVF-PQ trains coarse + per-list PQ codebooks (pq_idx.rs:357-396). */
int hora_build(hora_index *h, int metric);
int hora_built(const hora_index *h, int *out);         /* ann_index.rs:64 */
int hora_rebuild(hora_index *h, int metric);           /* ann_index.rs:69-71: ENOTIMPL */
/* search (ann_index.rs:91-97) for nq queries at once. */
int hora_search(hora_index *h, const float *queries, uint64_t nq, uint64_t k, uint64_t *ids_out,
                float *dist_out);
/* search_nodes (ann_index.rs:81-84): also copies each result's vector into
 * vecs_out (nq x k x dim; rows of missing results are zero). */
int hora_search_nodes(hora_index *h, const float *queries, uint64_t nq, uint64_t k,
                      uint64_t *ids_out, float *dist_out, float *vecs_out);
int hora_name(const hora_index *h, const char **out);  /* ann_index.rs:102 */
int hora_nodes_size(const hora_index *h, uint64_t *out); /* ann_index.rs:105-107 */
int hora_dimension(const hora_index *h, uint64_t *out);  /* ann_index.rs:118-120 */
int hora_clear(hora_index *h);                           /* ann_index.rs:110 */
/* idx_info (ann_index.rs:113-115): JSON statistics into buf (NUL-terminated). */
int hora_idx_info(const hora_index *h, char *buf, uint64_t cap);

/* ---- SerializableIndex (ann_index.rs:141-158) --------------------------- */
int hora_dump(hora_index *h, const char *path);
int hora_load(const char *path, hora_index **out);

/* ---- GPU options and parity hooks -------------------------------------- */
int hora_set_option(hora_index *h, int key, double value);
int hora_get_option(const hora_index *h, int key, double *out);

/* IVF-PQ layout, for inspection and for the parity tests.  Sizes:
 * centers n_list x dim; offsets n_list+1; items n (row numbers in insertion
 * order); codebooks n_list x n_sub x 2^sub_bits x dmax; codes n x n_sub in
 * list order; trained n_list.  dmax = dim/n_sub + (dim % (dim/n_sub) != 0).
 * Any output pointer may be NULL.  A PQIndex reports one list whose centre
 * is the zero vector (its codebooks are trained on the raw vectors). */
int hora_ivfpq_layout(const hora_index *h, uint64_t *n_list, uint64_t *n_sub,
                      uint64_t *sub_bits, uint64_t *dmax);
int hora_ivfpq_export(const hora_index *h, float *centers, int64_t *offsets, int64_t *items,
                      float *codebooks, uint8_t *codes, uint8_t *trained);
/* Replace the trained structure with given coarse centres and codebooks
 * (host memory): items are re-assigned to lists and re-encoded on the GPU.
 * The parity hook for "PQ codes bit-exact given identical codebooks". */
int hora_ivfpq_set_codebooks(hora_index *h, const float *centers, const float *codebooks);

/* SerializableIndex::load (ann_index.rs:141-158) of a file the reference
 * itself wrote with bincode (bruteforce_idx.rs:84-106, pq_idx.rs:243-265,
 * 488-523), for BruteForceIndex / PQIndex / IVFPQIndex<f32, usize> (kind
 * names the struct: bincode carries no type tag).  Vectors and ids are
 * added; a trained PQ / IVF-PQ index takes the file's coarse centres and
 * codebooks, its lists and codes are recomputed on the GPU and the lists are
 * checked against the file's.  sub_bits above 8 is HORA_ECAP. */
int hora_load_reference(const char *path, int kind, hora_index **out);

/* SSGIndex::build_knn_graph (src/index/ssg_idx.rs:69-98) on a built
 * BruteForceIndex: for every stored row, the row numbers of its k nearest
 * other rows under the index metric, in the reference's order (max-heap pop
 * order: farthest first).  Runs the brute-force search with the base's rows
 * as queries, in the index's precision.  neighbors_out: n x k (host). */
int hora_knn_graph(hora_index *h, uint64_t k, uint64_t *neighbors_out);

/* kmeans::general_kmeans (src/core/kmeans.rs:216-289; SSG's root selection,
 * src/index/ssg_idx.rs:388) over the rows of a built BruteForceIndex, with
 * the index metric.  The k means start as copies of the rows init_rows[0..k)
 * or, when init_rows is NULL, of k rows drawn with replacement from the
 * splitmix64 stream of `seed` (the reference draws from an unseeded thread
 * RNG); epoch rounds of nearest-mean assignment and f32 means (an empty mean
 * becomes NaN, as in the reference) follow.  roots_out (k, host): per mean,
 * the row number nearest to it; means_out (k x dim, host) may be NULL.
 * Writes nothing when the index holds no rows (the reference returns an empty
 * list).  k <= 32768, else HORA_ECAP. */
int hora_general_kmeans(hora_index *h, uint64_t k, uint64_t epoch, const uint64_t *init_rows,
                        uint64_t seed, uint64_t *roots_out, float *means_out);

/* Per-call nprobe override (search_n_center) for sweeps; 0 = the param. */
int hora_search_nprobe(hora_index *h, const float *queries, uint64_t nq, uint64_t k,
                       uint64_t nprobe, uint64_t *ids_out, float *dist_out);

/* ---- learned nprobe (GPU-only; no reference counterpart) ----------------- */
/* Generates labels on n_train training queries (host or device memory): the
 * smallest nprobe in the grid 1,2,4..max_nprobe whose top-10 reaches the
 * recall target against exact brute force (per query: with k = 10 a target
 * of 0.95 means all ten; a query no grid nprobe brings there takes the
 * smallest nprobe reaching its best recall), trains the MLP on the GPU with
 * the library's forward/backward kernels on the first nine tenths,
 * calibrates the margin on the last tenth (the smallest that keeps its
 * recall@10 at or above the target) and installs the model; hora_idx_info
 * reports the calibration.  stats_out (may be NULL) receives [final loss,
 * label mean, label max, epochs]. */
int hora_ivfpq_train_nprobe(hora_index *h, const float *train_queries, uint64_t n_train,
                            uint64_t max_nprobe, double recall_target, uint64_t epochs,
                            double *stats_out);
/* Feature vectors (n x 40) the model sees for each query; for tests. */
int hora_ivfpq_nprobe_features(hora_index *h, const float *queries, uint64_t nq,
                               float *features_out);
/* nprobe the model picks for each query (after margin and clamp). */
int hora_ivfpq_predict_nprobe(hora_index *h, const float *queries, uint64_t nq,
                              uint32_t *nprobe_out);

/* MLP kernels exposed for the gradient check (params packed as
 * [W1(h1 x f) b1 W2(h2 x h1) b2 W3(h2) b3]); all pointers host memory. */
int hora_mlp_forward(const float *params, uint64_t f, uint64_t h1, uint64_t h2,
                     const float *x, uint64_t n, float *out);
int hora_mlp_loss_grad(const float *params, uint64_t f, uint64_t h1, uint64_t h2,
                       const float *x, const float *y, uint64_t n, float alpha,
                       float *loss_out, float *grad_out);

/* ---- serving (GPU-only; no reference counterpart) ------------------------ */
/* A continuous-batching request loop over one or more built indexes: requests
 * of any batch size and k are submitted from any thread, admitted while the
 * bytes they need fit the HBM budget and a slot is free, and batched onto
 * the GPU streams as slots free up.  Latency per request is measured from
 * submit to completion. */
typedef struct hora_server hora_server;
int hora_server_create(hora_index *const *indexes, uint32_t n_indexes, uint32_t n_slots,
                       uint64_t hbm_budget_bytes, hora_server **out);
int hora_server_free(hora_server *s);
/* Queues a request; results land in the caller's host buffers (nq x k).
 * Returns a ticket > 0 in *ticket. */
int hora_server_submit(hora_server *s, uint32_t index_no, const float *queries, uint64_t nq,
                       uint64_t k, uint64_t *ids_out, float *dist_out, uint64_t *ticket);
/* Waits until the ticket completes (timeout_ms < 0: no limit). */
int hora_server_wait(hora_server *s, uint64_t ticket, int64_t timeout_ms, double *latency_ms);
/* Aggregate statistics: [completed requests, completed queries, p50 ms,
 * p99 ms, max in-flight requests, max admitted bytes, rejected]. */
int hora_server_stats(hora_server *s, double *out7);
/* The device bytes a request of nq queries at k is charged against the HBM
 * budget (an upper estimate of what its search reserves in a slot). */
int hora_server_request_bytes(hora_server *s, uint32_t index_no, uint64_t nq, uint64_t k,
                              uint64_t *out);
/* JSON diagnostics: batches run, batches that mixed different k, and the
 * device bytes each slot's search workspace holds. */
int hora_server_info(hora_server *s, char *buf, uint64_t cap);

/* ---- brute force without device allocation ------------------------------- */
/* No counterpart in the reference.  Exact brute-force k-NN for callers that
 * cannot call cudaMalloc (a host engine that owns all device memory through
 * its own pool and budget, or a latency-critical path where cudaMalloc /
 * cudaFree would synchronise the device).  base (n x dim), queries (nq x dim),
 * ids_out and dist_out (nq x k, row numbers and distances as hora_search
 * returns them) are all memory of the current device (or managed memory;
 * anything else is HORA_EINVAL); dim must be a multiple of 4 and the rows
 * 16-byte aligned.  A NaN or Inf element in the queries or the base is
 * HORA_ENAN (reported before any result is written).  Scratch comes from one
 * fixed 2.1 MiB device array that every GPU loading the library holds until
 * the process exits: at most 256 queries and k <= 64 per call (HORA_ECAP
 * beyond), metrics Euclidean, Manhattan and DotProduct.  Calls share that
 * array: calls that overlap on the GPU race.  The call is synchronous: it
 * returns once the results are in ids_out / dist_out.  The first call on each
 * device resolves the array's device address; make it before any stream
 * capture.  stream may be NULL. */
int hora_bf_search_noalloc(const float *base, uint64_t n, uint64_t dim, const float *queries,
                           uint64_t nq, uint64_t k, int metric, uint64_t *ids_out,
                           float *dist_out, void *stream);

/* ---- diagnostics -------------------------------------------------------- */
const char *hora_last_error(void);
const char *hora_version(void);
/* Number of kernels this library has launched in the process (for the
 * bench's launch count). */
uint64_t hora_kernel_launches(void);
/* Kernel timing: while enabled, every launch of the library is bracketed by
 * CUDA events on its own stream.  hora_profile_report synchronises, writes
 * {"kernel": [launches, total_ms], ...} as JSON into buf and clears. */
int hora_profile_enable(int on);
int hora_profile_report(char *buf, uint64_t cap);

#ifdef __cplusplus
}
#endif
#endif
