/*
 * hora_oracle.c — CPU restatement of hora's search path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libhora_gb300.so.  Loaded by
 * tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py; the
 * product never calls it.  Parity status per component is in hora_oracle.h.
 *
 * Compiled with -O2 -ffp-contract=off and no fast-math: Rust/LLVM never
 * contracts a*b+c into an FMA, so every f32 operation here rounds exactly
 * where the reference's scalar code rounds.
 */
#include "hora_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* distances — src/core/simd_metrics.rs:30-33 (dot), :60-66 (L1), :96-102 (L2)
 * scalar branches; src/core/metrics.rs:22-34 dispatch.                      */

float horo_calc_dot_f32(const float *a, const float *b, int64_t d) {
  /* simd_metrics.rs:32: Ok(-(a.iter().zip(b).map(|(p,q)| p*q).sum())) */
  float s = 0.0f;
  for (int64_t i = 0; i < d; ++i) s = s + a[i] * b[i];
  return -s;
}

double horo_calc_dot_f64(const double *a, const double *b, int64_t d) {
  double s = 0.0;
  for (int64_t i = 0; i < d; ++i) s = s + a[i] * b[i];
  return -s;
}

static float l2_f32(const float *a, const float *b, int64_t d) {
  float s = 0.0f;
  for (int64_t i = 0; i < d; ++i) {
    float t = a[i] - b[i];
    s = s + t * t; /* (p - q).powi(2) == t*t */
  }
  return s;
}

static float l1_f32(const float *a, const float *b, int64_t d) {
  float s = 0.0f;
  for (int64_t i = 0; i < d; ++i) s = s + fabsf(a[i] - b[i]);
  return s;
}

/* metrics.rs:50-57: dot_product(v1,v2) = -(calc::dot(v1,v2)) = +sum(p*q). */
static float ip_f32(const float *a, const float *b, int64_t d) {
  return -horo_calc_dot_f32(a, b, d);
}

/* metrics.rs:73-83 as intended: -(a.b)/(|a||b|).  A zero norm gives 0. */
static float cos_f32(const float *a, const float *b, int64_t d) {
  float ab = 0.0f, aa = 0.0f, bb = 0.0f;
  for (int64_t i = 0; i < d; ++i) ab = ab + a[i] * b[i];
  for (int64_t i = 0; i < d; ++i) aa = aa + a[i] * a[i];
  for (int64_t i = 0; i < d; ++i) bb = bb + b[i] * b[i];
  float den = sqrtf(aa) * sqrtf(bb);
  if (den == 0.0f) return 0.0f;
  return -ab / den;
}

float horo_metric_f32(const float *a, const float *b, int64_t d, int metric, int *err) {
  if (err) *err = 0;
  switch (metric) {
    case HORO_EUCLIDEAN: return l2_f32(a, b, d);
    case HORO_MANHATTAN: return l1_f32(a, b, d);
    case HORO_DOT: return ip_f32(a, b, d);
    case HORO_COSINE: return cos_f32(a, b, d);
    default:
      if (err) *err = 1; /* Result::Err("unknown method") */
      return 0.0f;
  }
}

double horo_metric_f64(const double *a, const double *b, int64_t d, int metric, int *err) {
  if (err) *err = 0;
  double s = 0.0;
  switch (metric) {
    case HORO_EUCLIDEAN:
      for (int64_t i = 0; i < d; ++i) { double t = a[i] - b[i]; s = s + t * t; }
      return s;
    case HORO_MANHATTAN:
      for (int64_t i = 0; i < d; ++i) s = s + fabs(a[i] - b[i]);
      return s;
    case HORO_DOT: return -horo_calc_dot_f64(a, b, d);
    case HORO_COSINE: {
      double ab = 0, aa = 0, bb = 0;
      for (int64_t i = 0; i < d; ++i) { ab += a[i] * b[i]; aa += a[i] * a[i]; bb += b[i] * b[i]; }
      double den = sqrt(aa) * sqrt(bb);
      return den == 0.0 ? 0.0 : -ab / den;
    }
    default:
      if (err) *err = 1;
      return 0.0;
  }
}

/* f64 accumulation of f32 inputs, for the exact oracle. */
static double metric_acc64(const float *a, const float *b, int64_t d, int metric) {
  double s = 0.0;
  switch (metric) {
    case HORO_EUCLIDEAN:
      for (int64_t i = 0; i < d; ++i) { double t = (double)a[i] - (double)b[i]; s += t * t; }
      return s;
    case HORO_MANHATTAN:
      for (int64_t i = 0; i < d; ++i) s += fabs((double)a[i] - (double)b[i]);
      return s;
    case HORO_DOT:
      for (int64_t i = 0; i < d; ++i) s += (double)a[i] * (double)b[i];
      return s;
    case HORO_COSINE: {
      double ab = 0, aa = 0, bb = 0;
      for (int64_t i = 0; i < d; ++i) {
        ab += (double)a[i] * b[i]; aa += (double)a[i] * a[i]; bb += (double)b[i] * b[i];
      }
      double den = sqrt(aa) * sqrt(bb);
      return den == 0.0 ? 0.0 : -ab / den;
    }
    default: return 0.0;
  }
}

/* ------------------------------------------------------------------------ */
/* std::collections::BinaryHeap<Neighbor> — max-heap on distance, with the
 * sift_up / sift_down_to_bottom order of the std implementation (the
 * reference's own copy is src/core/heap.rs:21-35,54-68,95-112).  Neighbor's
 * ordering compares distances only (src/core/neighbor.rs:30-34).           */

typedef struct { int64_t idx; float d; } nb_t;
typedef struct { nb_t *a; int64_t len, cap; } heap_t;

static void heap_init(heap_t *h, int64_t cap) {
  h->cap = cap > 4 ? cap : 4;
  h->len = 0;
  h->a = (nb_t *)malloc(sizeof(nb_t) * (size_t)h->cap);
}
static void heap_free(heap_t *h) { free(h->a); h->a = NULL; h->len = h->cap = 0; }

static void heap_sift_up(heap_t *h, int64_t start, int64_t pos) {
  nb_t e = h->a[pos];
  while (pos > start) {
    int64_t parent = (pos - 1) / 2;
    if (e.d <= h->a[parent].d) break;
    h->a[pos] = h->a[parent];
    pos = parent;
  }
  h->a[pos] = e;
}

static void heap_push(heap_t *h, nb_t x) {
  if (h->len == h->cap) {
    h->cap *= 2;
    h->a = (nb_t *)realloc(h->a, sizeof(nb_t) * (size_t)h->cap);
  }
  h->a[h->len++] = x;
  heap_sift_up(h, 0, h->len - 1);
}

static void heap_sift_down_to_bottom(heap_t *h, int64_t pos) {
  int64_t end = h->len, start = pos;
  nb_t e = h->a[pos];
  int64_t child = 2 * pos + 1;
  while (child + 1 < end) {
    child += (h->a[child].d <= h->a[child + 1].d) ? 1 : 0;
    h->a[pos] = h->a[child];
    pos = child;
    child = 2 * pos + 1;
  }
  if (child == end - 1) {
    h->a[pos] = h->a[child];
    pos = child;
  }
  h->a[pos] = e;
  heap_sift_up(h, start, pos);
}

static nb_t heap_pop(heap_t *h) {
  nb_t item = h->a[--h->len];
  if (h->len > 0) {
    nb_t top = h->a[0];
    h->a[0] = item;
    item = top;
    heap_sift_down_to_bottom(h, 0);
  }
  return item;
}

/* ------------------------------------------------------------------------ */
/* A small query-parallel for-loop over pthreads. */

typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi);
typedef struct { range_fn fn; void *ctx; int64_t lo, hi; } range_job;

static void *range_thread(void *p) {
  range_job *j = (range_job *)p;
  j->fn(j->ctx, j->lo, j->hi);
  return NULL;
}

static void parallel_for(int64_t n, int threads, range_fn fn, void *ctx) {
  if (threads <= 1 || n < 2) {
    fn(ctx, 0, n);
    return;
  }
  if (threads > n) threads = (int)n;
  pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  range_job *jobs = (range_job *)malloc(sizeof(range_job) * (size_t)threads);
  for (int t = 0; t < threads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].lo = n * t / threads;
    jobs[t].hi = n * (t + 1) / threads;
    pthread_create(&tid[t], NULL, range_thread, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
  free(tid);
  free(jobs);
}

/* ------------------------------------------------------------------------ */
/* BruteForceIndex::node_search_k — src/index/bruteforce_idx.rs:47-73.      */

typedef struct {
  const float *base, *queries;
  int64_t n, dim, k;
  int metric;
  int64_t *idx_out;
  float *dist_out;
} bf_ctx;

static void bf_range(void *p, int64_t lo, int64_t hi) {
  bf_ctx *c = (bf_ctx *)p;
  heap_t h;
  heap_init(&h, c->k + 2);
  nb_t *tmp = (nb_t *)malloc(sizeof(nb_t) * (size_t)(c->k + 1));
  for (int64_t qi = lo; qi < hi; ++qi) {
    const float *q = c->queries + qi * c->dim;
    h.len = 0;
    for (int64_t i = 0; i < c->n; ++i) {
      nb_t x = {i, horo_metric_f32(q, c->base + i * c->dim, c->dim, c->metric, NULL)};
      heap_push(&h, x); /* heap.push(Neighbor::new(i, item.metric(node))) */
      if (h.len > c->k) (void)heap_pop(&h); /* if heap.len() > k { heap.pop() } */
    }
    int64_t m = 0;
    while (h.len > 0) tmp[m++] = heap_pop(&h); /* pop all, then reverse */
    for (int64_t j = 0; j < c->k; ++j) {
      if (j < m) {
        c->idx_out[qi * c->k + j] = tmp[m - 1 - j].idx;
        c->dist_out[qi * c->k + j] = tmp[m - 1 - j].d;
      } else {
        c->idx_out[qi * c->k + j] = -1;
        c->dist_out[qi * c->k + j] = INFINITY;
      }
    }
  }
  free(tmp);
  heap_free(&h);
}

int horo_bf_search(const float *base, int64_t n, int64_t dim, const float *queries, int64_t nq,
                   int64_t k, int metric, int64_t *idx_out, float *dist_out, int threads) {
  if (metric != HORO_EUCLIDEAN && metric != HORO_MANHATTAN && metric != HORO_DOT &&
      metric != HORO_COSINE)
    return -1;
  bf_ctx c = {base, queries, n, dim, k, metric, idx_out, dist_out};
  parallel_for(nq, threads, bf_range, &c);
  return 0;
}

/* Exact f64 top-k, ties by index: bounded max-heap on (d, idx). */
typedef struct { int64_t idx; double d; } nb64_t;

static int nb64_less(nb64_t a, nb64_t b) { return a.d < b.d || (a.d == b.d && a.idx < b.idx); }

static void h64_sift_down(nb64_t *a, int64_t n, int64_t pos) {
  for (;;) {
    int64_t l = 2 * pos + 1, r = l + 1, big = pos;
    if (l < n && nb64_less(a[big], a[l])) big = l;
    if (r < n && nb64_less(a[big], a[r])) big = r;
    if (big == pos) return;
    nb64_t t = a[pos]; a[pos] = a[big]; a[big] = t;
    pos = big;
  }
}
static void h64_sift_up(nb64_t *a, int64_t pos) {
  while (pos > 0) {
    int64_t p = (pos - 1) / 2;
    if (!nb64_less(a[p], a[pos])) return;
    nb64_t t = a[pos]; a[pos] = a[p]; a[p] = t;
    pos = p;
  }
}

typedef struct {
  const float *base, *queries;
  int64_t n, dim, k;
  int metric;
  int64_t *idx_out;
  double *dist_out;
} bf64_ctx;

static int cmp_nb64(const void *x, const void *y) {
  nb64_t a = *(const nb64_t *)x, b = *(const nb64_t *)y;
  return nb64_less(a, b) ? -1 : (nb64_less(b, a) ? 1 : 0);
}

static void bf64_range(void *p, int64_t lo, int64_t hi) {
  bf64_ctx *c = (bf64_ctx *)p;
  nb64_t *h = (nb64_t *)malloc(sizeof(nb64_t) * (size_t)(c->k + 1));
  for (int64_t qi = lo; qi < hi; ++qi) {
    const float *q = c->queries + qi * c->dim;
    int64_t len = 0;
    for (int64_t i = 0; i < c->n; ++i) {
      nb64_t x = {i, metric_acc64(q, c->base + i * c->dim, c->dim, c->metric)};
      if (len < c->k) {
        h[len] = x;
        h64_sift_up(h, len);
        ++len;
      } else if (c->k > 0 && nb64_less(x, h[0])) {
        h[0] = x;
        h64_sift_down(h, len, 0);
      }
    }
    qsort(h, (size_t)len, sizeof(nb64_t), cmp_nb64);
    for (int64_t j = 0; j < c->k; ++j) {
      c->idx_out[qi * c->k + j] = j < len ? h[j].idx : -1;
      c->dist_out[qi * c->k + j] = j < len ? h[j].d : INFINITY;
    }
  }
  free(h);
}

int horo_bf_exact_f64(const float *base, int64_t n, int64_t dim, const float *queries,
                      int64_t nq, int64_t k, int metric, int64_t *idx_out, double *dist_out,
                      int threads) {
  bf64_ctx c = {base, queries, n, dim, k, metric, idx_out, dist_out};
  parallel_for(nq, threads, bf64_range, &c);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Seeded randomness replacing rand::thread_rng (src/core/kmeans.rs:168). */

static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint64_t horo_rng_instance_seed(uint64_t seed, uint64_t instance) {
  return mix64(seed ^ mix64(instance * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull));
}

uint64_t horo_rng_next(uint64_t *state) {
  *state += 0x9E3779B97F4A7C15ull;
  return mix64(*state);
}

double horo_rng_unit(uint64_t *state) {
  return (double)(horo_rng_next(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------------------ */
/* Kmeans — src/core/kmeans.rs:36-207.                                       */

static inline float kval(const float *row, int64_t col, const float *residual) {
  /* kmeans.rs:37-41,59-63,107-111: x[begin+j] - residual[begin+j] in f32 */
  return residual ? row[col] - residual[col] : row[col];
}

void horo_kmeans_init(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                      const float *residual, int64_t n_center, int accum_f64, float *centers) {
  int64_t dim = end - begin;
  float *mean = (float *)calloc((size_t)dim, sizeof(float));
  if (accum_f64) {
    double *s = (double *)calloc((size_t)dim, sizeof(double));
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < dim; ++j) s[j] += (double)kval(data + i * stride, begin + j, residual);
    for (int64_t j = 0; j < dim; ++j) mean[j] = (float)(s[j] / (double)n);
    free(s);
  } else {
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = 0; j < dim; ++j) mean[j] += kval(data + i * stride, begin + j, residual);
    for (int64_t j = 0; j < dim; ++j) mean[j] /= (float)n; /* E::from_usize(batch_size) */
  }
  /* kmeans.rs:72-84: `i & (1 << j) == 1` parses as (i & (1<<j)) == 1 and the
   * shift amount wraps at 64 (overflow-checks = false), so it holds only for
   * odd i and j % 64 == 0. */
  for (int64_t i = 0; i < n_center; ++i)
    for (int64_t j = 0; j < dim; ++j) {
      uint64_t bit = (uint64_t)1 << ((uint64_t)j & 63);
      int plus = (((uint64_t)i & bit) == 1);
      centers[i * dim + j] = plus ? mean[j] + 1.0f : mean[j] - 1.0f;
    }
  free(mean);
}

void horo_kmeans_assign(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                        const float *residual, const float *centers, int64_t n_center, int metric,
                        int64_t *assign_out) {
  int64_t dim = end - begin;
  float *z = (float *)malloc(sizeof(float) * (size_t)(dim > 0 ? dim : 1));
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t j = 0; j < dim; ++j) z[j] = kval(data + i * stride, begin + j, residual);
    /* kmeans.rs:135-146: strict '<' against the incumbent, starting at 0.  The
     * reference recomputes the incumbent distance on every compare; the value
     * is the same, so it is cached here. */
    int64_t best = 0;
    float bd = horo_metric_f32(z, centers, dim, metric, NULL);
    for (int64_t c = 1; c < n_center; ++c) {
      float d = horo_metric_f32(z, centers + c * dim, dim, metric, NULL);
      if (d < bd) { bd = d; best = c; }
    }
    assign_out[i] = best;
  }
  free(z);
}

void horo_kmeans_update(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                        const float *residual, const int64_t *assign, int64_t n_center,
                        int accum_f64, float *centers, int64_t *counts_out) {
  int64_t dim = end - begin;
  memset(counts_out, 0, sizeof(int64_t) * (size_t)n_center);
  if (accum_f64) {
    double *s = (double *)calloc((size_t)(n_center * dim), sizeof(double));
    for (int64_t i = 0; i < n; ++i) {
      int64_t c = assign[i];
      counts_out[c] += 1;
      for (int64_t j = 0; j < dim; ++j) s[c * dim + j] += (double)kval(data + i * stride, begin + j, residual);
    }
    for (int64_t c = 0; c < n_center; ++c)
      for (int64_t j = 0; j < dim; ++j)
        centers[c * dim + j] = counts_out[c] ? (float)(s[c * dim + j] / (double)counts_out[c]) : 0.0f;
    free(s);
  } else {
    /* kmeans.rs:97-124: f32 sums, divide by count, empty -> zero vector */
    memset(centers, 0, sizeof(float) * (size_t)(n_center * dim));
    for (int64_t i = 0; i < n; ++i) {
      int64_t c = assign[i];
      counts_out[c] += 1;
      for (int64_t j = 0; j < dim; ++j) centers[c * dim + j] += kval(data + i * stride, begin + j, residual);
    }
    for (int64_t c = 0; c < n_center; ++c) {
      if (counts_out[c] == 0) continue;
      for (int64_t j = 0; j < dim; ++j) centers[c * dim + j] /= (float)counts_out[c];
    }
  }
}

int horo_kmeans_split(float *centers, int64_t *counts, int64_t n_center, int64_t dim,
                      int64_t batch_size, uint64_t *rng_state) {
  /* kmeans.rs:150-193 */
  if (batch_size == 0) return -1; /* Err("None to assigned impossible split center") */
  const float eps = 1.0f / 1024.0f;
  const float lo = 1.0f - eps, hi = 1.0f + eps;
  for (int64_t i = 0; i < n_center; ++i) {
    if (counts[i] != 0) continue;
    int64_t s = (i + 1) % n_center;
    int64_t guard = 0;
    for (;;) {
      /* accept with probability p = counts[s] / batch_size: the draw u is a
       * 53-bit integer and u / 2^53 < counts / batch is tested exactly as
       * u * batch < counts * 2^53 (128-bit).  A draw at p == 0 can never
       * accept; both builds skip it. */
      if (counts[s] > 0) {
        uint64_t u = horo_rng_next(rng_state) >> 11;
        unsigned __int128 lhs = (unsigned __int128)u * (uint64_t)batch_size;
        unsigned __int128 rhs = (unsigned __int128)(uint64_t)counts[s] << 53;
        if (lhs < rhs) break;
      }
      s = (s + 1) % n_center;
      if (++guard > (int64_t)1 << 40) return -2;
    }
    for (int64_t j = 0; j < dim; ++j) {
      if (j % 2 == 0) {
        centers[i * dim + j] = centers[s * dim + j] * lo;
        centers[s * dim + j] *= hi;
      } else {
        centers[i * dim + j] = centers[s * dim + j] * hi;
        centers[s * dim + j] *= lo;
      }
    }
    counts[i] = counts[s] / 2;
    counts[s] -= counts[i];
  }
  return 0;
}

int horo_kmeans_train(const float *data, int64_t n, int64_t stride, int64_t begin, int64_t end,
                      const float *residual, int64_t n_center, int64_t n_epoch, int metric,
                      uint64_t rng_seed, int accum_f64, float *centers_out) {
  /* kmeans.rs:195-207 */
  uint64_t rng = rng_seed;
  horo_kmeans_init(data, n, stride, begin, end, residual, n_center, accum_f64, centers_out);
  int64_t *assign = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t *counts = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_center);
  int rc = 0;
  for (int64_t ep = 0; ep < n_epoch; ++ep) {
    horo_kmeans_assign(data, n, stride, begin, end, residual, centers_out, n_center, metric, assign);
    horo_kmeans_update(data, n, stride, begin, end, residual, assign, n_center, accum_f64, centers_out, counts);
    if (ep < n_epoch - 1) {
      rc = horo_kmeans_split(centers_out, counts, n_center, end - begin, n, &rng);
      if (rc) break;
    }
  }
  free(assign);
  free(counts);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* PQ / IVF-PQ — src/index/pq_idx.rs.                                        */

void horo_pq_ranges(int64_t dim, int64_t n_sub, int64_t *begin_out, int64_t *end_out) {
  /* pq_idx.rs:75-88 (uses dimension % sub_dimension as written) */
  int64_t sd = dim / n_sub;
  int64_t r = dim % sd;
  for (int64_t i = 0; i < n_sub; ++i) {
    if (i < r) {
      begin_out[i] = i * (sd + 1);
      end_out[i] = (i + 1) * (sd + 1);
    } else {
      begin_out[i] = r * (sd + 1) + (i - r) * sd;
      end_out[i] = r * (sd + 1) + (i + 1 - r) * sd;
    }
  }
}

static int64_t pq_dmax(int64_t dim, int64_t n_sub) {
  int64_t sd = dim / n_sub;
  return sd + ((dim % sd) ? 1 : 0);
}

void horo_pq_encode(const float *data, int64_t n, int64_t dim, const float *list_center,
                    const float *codebook, int64_t n_sub, int64_t sub_bits, uint8_t *codes_out) {
  int64_t K = (int64_t)1 << sub_bits, dmax = pq_dmax(dim, n_sub);
  int64_t *b = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  horo_pq_ranges(dim, n_sub, b, e);
  float *sub = (float *)malloc(sizeof(float) * (size_t)(K * dmax));
  int64_t *a = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  for (int64_t m = 0; m < n_sub; ++m) {
    int64_t len = e[m] - b[m];
    for (int64_t j = 0; j < K; ++j)
      for (int64_t t = 0; t < len; ++t) sub[j * len + t] = codebook[(m * K + j) * dmax + t];
    horo_kmeans_assign(data, n, dim, b[m], e[m], list_center, sub, K, HORO_EUCLIDEAN, a);
    for (int64_t i = 0; i < n; ++i) codes_out[i * n_sub + m] = (uint8_t)a[i];
  }
  free(a);
  free(sub);
  free(b);
  free(e);
}

void horo_pq_lut(const float *query, int64_t dim, const float *list_center, const float *codebook,
                 int64_t n_sub, int64_t sub_bits, float *lut_out) {
  /* pq_idx.rs:151-163,170-179: LUT[m*K+j] = L2(q[range]-residual[range], C[m][j]) */
  int64_t K = (int64_t)1 << sub_bits, dmax = pq_dmax(dim, n_sub);
  int64_t *b = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  horo_pq_ranges(dim, n_sub, b, e);
  float *z = (float *)malloc(sizeof(float) * (size_t)dmax);
  for (int64_t m = 0; m < n_sub; ++m) {
    int64_t len = e[m] - b[m];
    for (int64_t t = 0; t < len; ++t) z[t] = query[b[m] + t] - list_center[b[m] + t];
    for (int64_t j = 0; j < K; ++j) lut_out[m * K + j] = l2_f32(z, codebook + (m * K + j) * dmax, len);
  }
  free(z);
  free(b);
  free(e);
}

int horo_ivfpq_build(const float *data, int64_t n, int64_t dim, int64_t n_sub, int64_t sub_bits,
                     int64_t n_list, int64_t n_epoch, int metric, uint64_t seed, int accum_f64,
                     int64_t train_size, float *centers_out, int64_t *list_offsets_out,
                     int64_t *list_items_out, float *codebooks_out, uint8_t *codes_out,
                     uint8_t *list_trained_out) {
  if (n <= 0 || n_sub <= 0 || dim < n_sub || sub_bits < 1 || sub_bits > 8) return -1;
  int64_t T = (train_size > 0 && train_size < n) ? train_size : n;
  int64_t K = (int64_t)1 << sub_bits, dmax = pq_dmax(dim, n_sub);
  /* pq_idx.rs:362-368: coarse k-means over the (training) items */
  int rc = horo_kmeans_train(data, T, dim, 0, dim, NULL, n_list, n_epoch, metric,
                             horo_rng_instance_seed(seed, 0), accum_f64, centers_out);
  if (rc) return rc;
  /* pq_idx.rs:369-375: assign every item, lists in increasing item order */
  int64_t *assign = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  horo_kmeans_assign(data, n, dim, 0, dim, NULL, centers_out, n_list, metric, assign);
  memset(list_offsets_out, 0, sizeof(int64_t) * (size_t)(n_list + 1));
  for (int64_t i = 0; i < n; ++i) list_offsets_out[assign[i] + 1]++;
  for (int64_t c = 0; c < n_list; ++c) list_offsets_out[c + 1] += list_offsets_out[c];
  int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_list);
  memcpy(cur, list_offsets_out, sizeof(int64_t) * (size_t)n_list);
  for (int64_t i = 0; i < n; ++i) list_items_out[cur[assign[i]]++] = i;
  free(cur);
  free(assign);

  int64_t *b = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  horo_pq_ranges(dim, n_sub, b, e);
  memset(codebooks_out, 0, sizeof(float) * (size_t)(n_list * n_sub * K * dmax));
  memset(codes_out, 0, (size_t)(n * n_sub));
  float *rows = NULL;
  float *sub = (float *)malloc(sizeof(float) * (size_t)(K * dmax));
  int64_t *a = NULL;
  for (int64_t c = 0; c < n_list; ++c) {
    int64_t off = list_offsets_out[c], L = list_offsets_out[c + 1] - off;
    list_trained_out[c] = 0;
    if (L == 0) continue; /* the reference panics here (kmeans.rs:158-160) */
    rows = (float *)realloc(rows, sizeof(float) * (size_t)(L * dim));
    a = (int64_t *)realloc(a, sizeof(int64_t) * (size_t)L);
    int64_t nt = 0;
    for (int64_t i = 0; i < L; ++i)
      if (list_items_out[off + i] < T) nt++;
    /* training rows: members among the training items, else all members */
    int64_t w = 0;
    for (int64_t i = 0; i < L; ++i) {
      int64_t it = list_items_out[off + i];
      if (nt == 0 || it < T) memcpy(rows + (w++) * dim, data + it * dim, sizeof(float) * (size_t)dim);
    }
    for (int64_t m = 0; m < n_sub; ++m) {
      int64_t len = e[m] - b[m];
      /* pq_idx.rs:136-142 */
      rc = horo_kmeans_train(rows, w, dim, b[m], e[m], centers_out + c * dim, K, n_epoch,
                             HORO_EUCLIDEAN, horo_rng_instance_seed(seed, 1 + c * n_sub + m),
                             accum_f64, sub);
      if (rc) goto done;
      for (int64_t j = 0; j < K; ++j)
        for (int64_t t = 0; t < len; ++t)
          codebooks_out[((c * n_sub + m) * K + j) * dmax + t] = sub[j * len + t];
    }
    /* pq_idx.rs:143-144: codes of every member against the final codebook */
    for (int64_t i = 0; i < L; ++i)
      memcpy(rows + i * dim, data + list_items_out[off + i] * dim, sizeof(float) * (size_t)dim);
    horo_pq_encode(rows, L, dim, centers_out + c * dim, codebooks_out + c * n_sub * K * dmax, n_sub,
                   sub_bits, codes_out + off * n_sub);
    list_trained_out[c] = 1;
  }
done:
  free(rows);
  free(sub);
  free(a);
  free(b);
  free(e);
  return rc;
}

void horo_ivf_coarse(const float *centers, int64_t n_list, int64_t dim, int metric,
                     const float *query, float *dist_out) {
  for (int64_t i = 0; i < n_list; ++i)
    dist_out[i] = horo_metric_f32(query, centers + i * dim, dim, metric, NULL);
}

typedef struct {
  const float *centers, *codebooks, *queries;
  const int64_t *offs, *items;
  const uint8_t *codes, *trained;
  int64_t n_list, dim, n_sub, sub_bits, k, nprobe;
  int metric;
  int64_t *idx_out;
  float *dist_out;
} ivf_ctx;

static void ivf_range(void *p, int64_t lo, int64_t hi) {
  ivf_ctx *c = (ivf_ctx *)p;
  int64_t K = (int64_t)1 << c->sub_bits, dmax = pq_dmax(c->dim, c->n_sub);
  float *lut = (float *)malloc(sizeof(float) * (size_t)(c->n_sub * K));
  heap_t top_centers, top_cand, list_heap;
  heap_init(&top_centers, c->n_list + 1);
  heap_init(&top_cand, c->k + 2);
  heap_init(&list_heap, 1024);
  nb_t *tmp = (nb_t *)malloc(sizeof(nb_t) * (size_t)(c->k + 1));
  int64_t np = c->nprobe < c->n_list ? c->nprobe : c->n_list;
  for (int64_t qi = lo; qi < hi; ++qi) {
    const float *q = c->queries + qi * c->dim;
    top_centers.len = 0;
    top_cand.len = 0;
    /* pq_idx.rs:416-421: push Neighbor(i, -metric(q, c_i)) */
    for (int64_t i = 0; i < c->n_list; ++i) {
      nb_t x = {i, -horo_metric_f32(q, c->centers + i * c->dim, c->dim, c->metric, NULL)};
      heap_push(&top_centers, x);
    }
    for (int64_t pr = 0; pr < np; ++pr) {
      int64_t center = heap_pop(&top_centers).idx;
      if (!c->trained[center]) continue;
      int64_t off = c->offs[center], L = c->offs[center + 1] - off;
      horo_pq_lut(q, c->dim, c->centers + center * c->dim, c->codebooks + center * c->n_sub * K * dmax,
                  c->n_sub, c->sub_bits, lut);
      /* pq_idx.rs:181-191: push every item, then pop down to k */
      list_heap.len = 0;
      for (int64_t i = 0; i < L; ++i) {
        float d = 0.0f;
        const uint8_t *code = c->codes + (off + i) * c->n_sub;
        for (int64_t m = 0; m < c->n_sub; ++m) d += lut[m * K + code[m]];
        nb_t x = {i, d};
        heap_push(&list_heap, x);
      }
      while (list_heap.len > c->k) (void)heap_pop(&list_heap);
      /* pq_idx.rs:429-436: remap local -> global and bounded merge */
      while (list_heap.len > 0) {
        nb_t r = heap_pop(&list_heap);
        r.idx = c->items[off + r.idx];
        heap_push(&top_cand, r);
        if (top_cand.len > c->k) (void)heap_pop(&top_cand);
      }
    }
    int64_t m = 0;
    while (top_cand.len > 0) tmp[m++] = heap_pop(&top_cand);
    for (int64_t j = 0; j < c->k; ++j) {
      c->idx_out[qi * c->k + j] = j < m ? tmp[m - 1 - j].idx : -1;
      c->dist_out[qi * c->k + j] = j < m ? tmp[m - 1 - j].d : INFINITY;
    }
  }
  free(tmp);
  free(lut);
  heap_free(&top_centers);
  heap_free(&top_cand);
  heap_free(&list_heap);
}

int horo_ivfpq_search(const float *centers, int64_t n_list, int64_t dim,
                      const int64_t *list_offsets, const int64_t *list_items,
                      const float *codebooks, const uint8_t *codes, const uint8_t *list_trained,
                      int64_t n_sub, int64_t sub_bits, int metric, const float *queries,
                      int64_t nq, int64_t k, int64_t nprobe, int64_t *idx_out, float *dist_out,
                      int threads) {
  ivf_ctx c = {centers, codebooks, queries, list_offsets, list_items, codes, list_trained,
               n_list, dim, n_sub, sub_bits, k, nprobe, metric, idx_out, dist_out};
  parallel_for(nq, threads, ivf_range, &c);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Flat PQIndex — src/index/pq_idx.rs:21-265.  No residual; the build metric
 * drives both the k-means (train_center, pq_idx.rs:122-149) and the LUT
 * (get_distance_from_vec_range, pq_idx.rs:151-163).                       */

int horo_pq_build(const float *data, int64_t n, int64_t dim, int64_t n_sub, int64_t sub_bits,
                  int64_t n_epoch, int metric, uint64_t seed, int accum_f64, int64_t train_size,
                  float *codebooks_out, uint8_t *codes_out) {
  if (n <= 0 || n_sub <= 0 || dim < n_sub || sub_bits < 1 || sub_bits > 8) return -1;
  int64_t T = (train_size > 0 && train_size < n) ? train_size : n;
  int64_t K = (int64_t)1 << sub_bits, dmax = pq_dmax(dim, n_sub);
  int64_t *b = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_sub);
  horo_pq_ranges(dim, n_sub, b, e);
  memset(codebooks_out, 0, sizeof(float) * (size_t)(n_sub * K * dmax));
  float *sub = (float *)malloc(sizeof(float) * (size_t)(K * dmax));
  int64_t *a = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int rc = 0;
  for (int64_t m = 0; m < n_sub; ++m) {
    int64_t len = e[m] - b[m];
    /* pq_idx.rs:136-141: Kmeans::new(.., self.mt), train on the items */
    rc = horo_kmeans_train(data, T, dim, b[m], e[m], NULL, K, n_epoch, metric,
                           horo_rng_instance_seed(seed, 1 + m), accum_f64, sub);
    if (rc) break;
    for (int64_t j = 0; j < K; ++j)
      for (int64_t t = 0; t < len; ++t) codebooks_out[(m * K + j) * dmax + t] = sub[j * len + t];
    /* pq_idx.rs:143-144: search_data with the same metric */
    horo_kmeans_assign(data, n, dim, b[m], e[m], NULL, sub, K, metric, a);
    for (int64_t i = 0; i < n; ++i) codes_out[i * n_sub + m] = (uint8_t)a[i];
  }
  free(a);
  free(sub);
  free(b);
  free(e);
  return rc;
}

typedef struct {
  const float *codebooks, *queries;
  const uint8_t *codes;
  int64_t n, dim, n_sub, sub_bits, k;
  int metric;
  int64_t *idx_out;
  float *dist_out;
} pq_ctx;

static void pq_range(void *p, int64_t lo, int64_t hi) {
  pq_ctx *c = (pq_ctx *)p;
  int64_t K = (int64_t)1 << c->sub_bits, dmax = pq_dmax(c->dim, c->n_sub);
  int64_t *b = (int64_t *)malloc(sizeof(int64_t) * (size_t)c->n_sub);
  int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (size_t)c->n_sub);
  horo_pq_ranges(c->dim, c->n_sub, b, e);
  float *lut = (float *)malloc(sizeof(float) * (size_t)(c->n_sub * K));
  nb_t *tmp = (nb_t *)malloc(sizeof(nb_t) * (size_t)(c->k + 1));
  heap_t top;
  heap_init(&top, 1024);
  for (int64_t qi = lo; qi < hi; ++qi) {
    const float *q = c->queries + qi * c->dim;
    /* pq_idx.rs:170-179: LUT[m*K+j] = metric(q[range_m], C[m][j]) */
    for (int64_t m = 0; m < c->n_sub; ++m)
      for (int64_t j = 0; j < K; ++j)
        lut[m * K + j] = horo_metric_f32(q + b[m], c->codebooks + (m * K + j) * dmax, e[m] - b[m],
                                         c->metric, NULL);
    /* pq_idx.rs:181-193: push every item, pop down to k */
    top.len = 0;
    for (int64_t i = 0; i < c->n; ++i) {
      float d = 0.0f;
      const uint8_t *code = c->codes + i * c->n_sub;
      for (int64_t m = 0; m < c->n_sub; ++m) d += lut[m * K + code[m]];
      nb_t x = {i, d};
      heap_push(&top, x);
    }
    while (top.len > c->k) (void)heap_pop(&top);
    int64_t m = 0;
    while (top.len > 0) tmp[m++] = heap_pop(&top);
    for (int64_t j = 0; j < c->k; ++j) {
      c->idx_out[qi * c->k + j] = j < m ? tmp[m - 1 - j].idx : -1;
      c->dist_out[qi * c->k + j] = j < m ? tmp[m - 1 - j].d : INFINITY;
    }
  }
  heap_free(&top);
  free(tmp);
  free(lut);
  free(b);
  free(e);
}

int horo_pq_search(const float *codebooks, const uint8_t *codes, int64_t n, int64_t dim,
                   int64_t n_sub, int64_t sub_bits, int metric, const float *queries, int64_t nq,
                   int64_t k, int64_t *idx_out, float *dist_out, int threads) {
  pq_ctx c = {codebooks, queries, codes, n, dim, n_sub, sub_bits, k, metric, idx_out, dist_out};
  parallel_for(nq, threads, pq_range, &c);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* kmeans::general_kmeans — src/core/kmeans.rs:216-289.                      */

typedef struct {
  const float *rows;  /* the side scanned: nodes (assignment) or nodes (roots) */
  const float *means;
  int64_t n, dim, k;
  int metric, roots; /* roots: per mean the nearest node, else per node the nearest mean */
  int64_t *out;
} gk_ctx;

static void gk_range(void *arg, int64_t lo, int64_t hi) {
  const gk_ctx *c = (const gk_ctx *)arg;
  for (int64_t t = lo; t < hi; ++t) {
    /* kmeans.rs:240-247 and :276-283: index 0, distance E::max_value(),
     * strict '<', metric(node, mean) */
    int64_t idx = 0;
    float dist = FLT_MAX;
    const int64_t m = c->roots ? c->n : c->k;
    for (int64_t i = 0; i < m; ++i) {
      const float *node = c->roots ? c->rows + i * c->dim : c->rows + t * c->dim;
      const float *mean = c->roots ? c->means + t * c->dim : c->means + i * c->dim;
      float d = horo_metric_f32(node, mean, c->dim, c->metric, NULL);
      if (d < dist) {
        idx = i;
        dist = d;
      }
    }
    c->out[t] = idx;
  }
}

int horo_general_kmeans(const float *data, int64_t n, int64_t dim, int64_t k, int64_t epoch, int metric,
                        const int64_t *init_rows, uint64_t seed, int64_t *roots_out, float *means_out,
                        int threads) {
  if (n == 0) return 0; /* kmeans.rs:222-224: no roots */
  float *means = means_out;
  /* kmeans.rs:228-230: k rows drawn with replacement (seeded stream here) */
  uint64_t st = horo_rng_instance_seed(seed, 0);
  for (int64_t i = 0; i < k; ++i) {
    int64_t r;
    if (init_rows) {
      r = init_rows[i];
    } else {
      uint64_t u = horo_rng_next(&st);
      r = (int64_t)(((unsigned __int128)u * (uint64_t)n) >> 64);
    }
    if (r < 0 || r >= n) return -1;
    memcpy(means + i * dim, data + r * dim, sizeof(float) * (size_t)dim);
  }
  int64_t *asg = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)k);
  float *feat = (float *)malloc(sizeof(float) * (size_t)(k * dim));
  for (int64_t ep = 0; ep < epoch; ++ep) {
    gk_ctx c = {data, means, n, dim, k, metric, 0, asg};
    parallel_for(n, threads, gk_range, &c);
    /* kmeans.rs:248-254: f32 sums per mean, here in node order */
    memset(cnt, 0, sizeof(int64_t) * (size_t)k);
    memset(feat, 0, sizeof(float) * (size_t)(k * dim));
    for (int64_t j = 0; j < n; ++j) {
      float *f = feat + asg[j] * dim;
      for (int64_t t = 0; t < dim; ++t) f[t] += data[j * dim + t];
      cnt[asg[j]] += 1;
    }
    /* kmeans.rs:257-270: divide by the count (0 / 0 = NaN for an empty mean) */
    for (int64_t i = 0; i < k; ++i)
      for (int64_t t = 0; t < dim; ++t) means[i * dim + t] = feat[i * dim + t] / (float)cnt[i];
  }
  gk_ctx c = {data, means, n, dim, k, metric, 1, roots_out};
  parallel_for(k, threads, gk_range, &c);
  free(asg);
  free(cnt);
  free(feat);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* MLP oracle for the learned-nprobe gradient check (new; no reference
 * counterpart).  Double precision throughout.                              */

void horo_mlp_forward(const float *P, int64_t f, int64_t h1, int64_t h2, const float *x,
                      int64_t n, float *out) {
  const float *W1 = P, *b1 = W1 + h1 * f, *W2 = b1 + h1, *b2 = W2 + h2 * h1, *W3 = b2 + h2,
              *b3 = W3 + h2;
  double *a1 = (double *)malloc(sizeof(double) * (size_t)h1);
  double *a2 = (double *)malloc(sizeof(double) * (size_t)h2);
  for (int64_t i = 0; i < n; ++i) {
    const float *xi = x + i * f;
    for (int64_t u = 0; u < h1; ++u) {
      double s = b1[u];
      for (int64_t t = 0; t < f; ++t) s += (double)W1[u * f + t] * xi[t];
      a1[u] = s > 0 ? s : 0;
    }
    for (int64_t u = 0; u < h2; ++u) {
      double s = b2[u];
      for (int64_t t = 0; t < h1; ++t) s += (double)W2[u * h1 + t] * a1[t];
      a2[u] = s > 0 ? s : 0;
    }
    double o = b3[0];
    for (int64_t t = 0; t < h2; ++t) o += (double)W3[t] * a2[t];
    out[i] = (float)o;
  }
  free(a1);
  free(a2);
}

double horo_mlp_loss_grad(const float *P, int64_t f, int64_t h1, int64_t h2, const float *x,
                          const float *y, int64_t n, float alpha, double *g) {
  const float *W1 = P, *b1 = W1 + h1 * f, *W2 = b1 + h1, *b2 = W2 + h2 * h1, *W3 = b2 + h2,
              *b3 = W3 + h2;
  int64_t np = h1 * f + h1 + h2 * h1 + h2 + h2 + 1;
  memset(g, 0, sizeof(double) * (size_t)np);
  double *gW1 = g, *gb1 = gW1 + h1 * f, *gW2 = gb1 + h1, *gb2 = gW2 + h2 * h1, *gW3 = gb2 + h2,
         *gb3 = gW3 + h2;
  double *z1 = (double *)malloc(sizeof(double) * (size_t)h1);
  double *a1 = (double *)malloc(sizeof(double) * (size_t)h1);
  double *z2 = (double *)malloc(sizeof(double) * (size_t)h2);
  double *a2 = (double *)malloc(sizeof(double) * (size_t)h2);
  double *d2 = (double *)malloc(sizeof(double) * (size_t)h2);
  double *d1 = (double *)malloc(sizeof(double) * (size_t)h1);
  double loss = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const float *xi = x + i * f;
    for (int64_t u = 0; u < h1; ++u) {
      double s = b1[u];
      for (int64_t t = 0; t < f; ++t) s += (double)W1[u * f + t] * xi[t];
      z1[u] = s;
      a1[u] = s > 0 ? s : 0;
    }
    for (int64_t u = 0; u < h2; ++u) {
      double s = b2[u];
      for (int64_t t = 0; t < h1; ++t) s += (double)W2[u * h1 + t] * a1[t];
      z2[u] = s;
      a2[u] = s > 0 ? s : 0;
    }
    double o = b3[0];
    for (int64_t t = 0; t < h2; ++t) o += (double)W3[t] * a2[t];
    double r = o - (double)y[i];
    double w = (o < (double)y[i]) ? (double)alpha : 1.0;
    loss += w * r * r;
    double dout = 2.0 * w * r / (double)n;
    gb3[0] += dout;
    for (int64_t t = 0; t < h2; ++t) {
      gW3[t] += dout * a2[t];
      d2[t] = z2[t] > 0 ? dout * W3[t] : 0.0;
    }
    for (int64_t u = 0; u < h2; ++u) {
      gb2[u] += d2[u];
      for (int64_t t = 0; t < h1; ++t) gW2[u * h1 + t] += d2[u] * a1[t];
    }
    for (int64_t t = 0; t < h1; ++t) {
      double s = 0;
      for (int64_t u = 0; u < h2; ++u) s += d2[u] * W2[u * h1 + t];
      d1[t] = z1[t] > 0 ? s : 0.0;
    }
    for (int64_t u = 0; u < h1; ++u) {
      gb1[u] += d1[u];
      for (int64_t t = 0; t < f; ++t) gW1[u * f + t] += d1[u] * xi[t];
    }
  }
  free(z1); free(a1); free(z2); free(a2); free(d2); free(d1);
  return loss / (double)n;
}
