// api.cu — the C ABI (include/hora_gb300.h): index handles, add / build /
// search, serialization, options.  Mirrors trait ANNIndex and
// SerializableIndex (src/core/ann_index.rs:25-158).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "index.h"

namespace hora {

static thread_local std::string t_err;
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_profile{0};

namespace {
struct ProfRec {
  std::string name;
  cudaEvent_t a, b;
};
std::mutex g_prof_mu;
std::vector<ProfRec> g_prof;
}  // namespace

void prof_record(const char *name, cudaEvent_t a, cudaEvent_t b) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_prof.push_back({name, a, b});
}

void set_error(const std::string &msg) { t_err = msg; }
int fail(int code, const std::string &msg) {
  t_err = msg;
  return code;
}

int pointer_kind(const void *p) {
  if (!p) return PTR_HOST;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PTR_HOST;
  }
  if (a.type == cudaMemoryTypeManaged) return PTR_DEVICE;
  if (a.type != cudaMemoryTypeDevice) return PTR_HOST;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PTR_FOREIGN;
  }
  return a.device == dev ? PTR_DEVICE : PTR_FOREIGN;
}

bool is_device_ptr(const void *p) { return pointer_kind(p) == PTR_DEVICE; }

int check_not_foreign(const void *p, const char *what) {
  if (p && pointer_kind(p) == PTR_FOREIGN)
    return fail(HORA_EINVAL, std::string(what) + " is memory of another device");
  return HORA_OK;
}

int ensure_smem_attr(const void *kernel, int bytes) {
  if (bytes <= 48 * 1024) return HORA_OK;
  int dev = 0;
  HORA_CUDA_TRY(cudaGetDevice(&dev));
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> have;
  std::lock_guard<std::mutex> g(mu);
  int &cur = have[{kernel, dev}];
  if (cur >= bytes) return HORA_OK;
  HORA_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  cur = bytes;
  return HORA_OK;
}

const char *metric_name(int m) {
  switch (m) {
    case M_L1: return "Manhattan";
    case M_IP: return "DotProduct";
    case M_L2: return "Euclidean";
    case M_COS: return "CosineSimilarity";
    case HORA_METRIC_ANGULAR: return "Angular";
  }
  return "Unknown";
}

static bool metric_supported(int m) { return m == M_L1 || m == M_IP || m == M_L2 || m == M_COS; }

BaseView base_view(hora_index *h) {
  BaseView b;
  b.X = h->base.as<float>();
  b.n = h->n;
  b.ld = (int64_t)h->ld;
  b.dim = (int64_t)h->dim;
  b.xnorm = h->xnorm.as<float>();
  return b;
}

int ensure_norms(hora_index *h, cudaStream_t s) {
  if (h->norms_valid) return HORA_OK;
  HORA_TRY(h->xnorm.reserve(sizeof(float) * std::max<int64_t>(h->n, 1)));
  HORA_TRY(h->xsq64.reserve(sizeof(double) * std::max<int64_t>(h->n, 1)));
  HORA_TRY(launch_row_norms(h->base.as<float>(), h->n, h->ld, h->dim, h->xnorm.as<float>(),
                            h->xsq64.as<double>(), s));
  h->norms_valid = true;
  return HORA_OK;
}

// Host-side finiteness check (Node::new panics on NaN/Inf, node.rs:158-166).
static bool host_all_finite(const float *x, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

static int check_device_finite(const float *X, int64_t n, int64_t ld, int64_t dim, DevBuf &tmp,
                               cudaStream_t s) {
  HORA_TRY(tmp.reserve(sizeof(uint32_t)));
  HORA_CUDA_TRY(cudaMemsetAsync(tmp.ptr, 0, sizeof(uint32_t), s));
  HORA_TRY(launch_check_finite(X, n, ld, dim, tmp.as<uint32_t>(), s));
  uint32_t flag = 0;
  HORA_CUDA_TRY(cudaMemcpyAsync(&flag, tmp.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag) return fail(HORA_ENAN, "invalid float element");
  return HORA_OK;
}

int stage_queries(hora_index *h, const float *queries, int64_t nq, SearchWorkspace &ws,
                  cudaStream_t s, bool defer_check) {
  const bool dev = is_device_ptr(queries);
  if (!dev && !defer_check && !host_all_finite(queries, nq * (int64_t)h->dim))
    return fail(HORA_ENAN, "invalid float element");
  HORA_TRY(ws.q.reserve(sizeof(float) * nq * h->ld));
  // host queries come over in one pitched copy and are staged in place;
  // device queries are read where they are
  if (!dev)
    HORA_CUDA_TRY(cudaMemcpy2DAsync(ws.q.ptr, h->ld * 4, queries, h->dim * 4, h->dim * 4, nq,
                                    cudaMemcpyHostToDevice, s));
  float *qn = nullptr;
  double *qsq = nullptr;
  if (h->metric == M_COS || h->precision != HORA_PREC_FP32 || exact_tc_eligible(h, 1) || coarse_tc_eligible(h)) {
    HORA_TRY(ws.qnorm.reserve(sizeof(float) * nq + sizeof(double) * nq + 16));
    qn = ws.qnorm.as<float>();
    qsq = reinterpret_cast<double *>(ws.qnorm.as<char>() + round_up(sizeof(float) * nq, 16));
  }
  uint32_t *flag = nullptr;
  if (defer_check || dev) {
    HORA_TRY(ws.d_status.reserve(sizeof(uint32_t)));
    flag = ws.d_status.as<uint32_t>();
    HORA_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(uint32_t), s));
  }
  HORA_TRY(launch_stage_rows(dev ? queries : ws.q.as<float>(), dev ? h->dim : h->ld, nq, h->dim, h->ld,
                             ws.q.as<float>(), flag, qn, qsq, s));
  if (defer_check) {
    HORA_TRY(ws.h_status.reserve(sizeof(uint32_t)));
    HORA_TRY(ws.ev_status.ensure());
    HORA_CUDA_TRY(cudaMemcpyAsync(ws.h_status.ptr, flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaEventRecord(ws.ev_status.ev, s));
    ws.status_pending = true;
  } else if (dev) {
    uint32_t bad = 0;
    HORA_CUDA_TRY(cudaMemcpyAsync(&bad, flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    if (bad) return fail(HORA_ENAN, "invalid float element");
  }
  return HORA_OK;
}

int bf_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                   cudaStream_t s) {
  const bool xtc = exact_tc_eligible(h, k);
  if (h->metric == M_COS || h->precision != HORA_PREC_FP32 || xtc) HORA_TRY(ensure_norms(h, s));
  if (h->precision != HORA_PREC_FP32) return lowp_search_keys(h, nq, k, ws, d_best, s);
  if (xtc) return exact_tc_search_keys(h, nq, k, ws, d_best, s);
  int retries = 0;
  HORA_TRY(bf_topk_exact(base_view(h), h->metric, ws.q.as<float>(), ws.qnorm.as<float>(), nq, k,
                         h->cand_cap, ws, d_best, s, &retries));
  h->last_retries = retries;
  return HORA_OK;
}

int prepare_for_concurrent_search(hora_index *h) {
  std::lock_guard<std::mutex> g(h->mu);
  if (!h->built) return fail(HORA_ENOTBUILT, "index not built");
  cudaStream_t s = h->stream;
  if (h->metric == M_COS || h->precision != HORA_PREC_FP32) HORA_TRY(ensure_norms(h, s));
  if (h->kind == HORA_INDEX_BRUTE_FORCE && h->precision != HORA_PREC_FP32 && h->metric != M_L1)
    HORA_TRY(lowp_prepare(h, s));
  if (h->kind == HORA_INDEX_BRUTE_FORCE && exact_tc_eligible(h, 1)) {
    HORA_TRY(ensure_norms(h, s));
    HORA_TRY(exact_tc_prepare(h, s));
  }
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  return HORA_OK;
}

}  // namespace hora

using namespace hora;

// ============================================================================
extern "C" {

const char *hora_last_error(void) { return t_err.c_str(); }
const char *hora_version(void) { return "hora_gb300 0.1.0 (sm_103a)"; }
uint64_t hora_kernel_launches(void) { return g_launches.load(); }

int hora_profile_enable(int on) {
  g_profile.store(on ? 1 : 0);
  return HORA_OK;
}

int hora_profile_report(char *buf, uint64_t cap) {
  std::vector<ProfRec> recs;
  {
    std::lock_guard<std::mutex> g(g_prof_mu);
    recs.swap(g_prof);
  }
  std::vector<std::pair<std::string, std::pair<uint64_t, double>>> agg;
  for (auto &r : recs) {
    cudaEventSynchronize(r.b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
    bool found = false;
    for (auto &x : agg)
      if (x.first == r.name) {
        x.second.first += 1;
        x.second.second += ms;
        found = true;
      }
    if (!found) agg.push_back({r.name, {1, (double)ms}});
  }
  std::string s = "{";
  for (size_t i = 0; i < agg.size(); ++i) {
    char tmp[256];
    std::snprintf(tmp, sizeof(tmp), "%s\"%s\": [%llu, %.6f]", i ? ", " : "", agg[i].first.c_str(),
                  (unsigned long long)agg[i].second.first, agg[i].second.second);
    s += tmp;
  }
  s += "}";
  if (!buf || cap == 0) return fail(HORA_EINVAL, "null buffer");
  std::snprintf(buf, cap, "%s", s.c_str());
  return s.size() + 1 > cap ? fail(HORA_ECAP, "buffer too small") : HORA_OK;
}

void hora_ivfpq_params_default(hora_ivfpq_params *p) {
  if (!p) return;
  // IVFPQParams::default (src/index/pq_params.rs:80-91)
  p->n_sub = 25;
  p->sub_bits = 4;
  p->n_kmeans_center = 256;
  p->search_n_center = 8;
  p->train_epoch = 100;
}

void hora_pq_params_default(hora_pq_params *p) {
  if (!p) return;
  // PQParams::default (src/index/pq_params.rs:32-41)
  p->n_sub = 4;
  p->sub_bits = 4;
  p->train_epoch = 100;
}

int hora_index_create(int kind, uint64_t dim, const void *params, hora_index **out) {
  if (!out) return fail(HORA_EINVAL, "out is null");
  *out = nullptr;
  if (kind != HORA_INDEX_BRUTE_FORCE && kind != HORA_INDEX_IVFPQ && kind != HORA_INDEX_PQ)
    return fail(HORA_EINVAL, "unknown index kind");
  if (dim == 0) return fail(HORA_EINVAL, "dimension must be positive");
  if (dim >= (1ull << 20)) return fail(HORA_ECAP, "dimension too large");
  hora_index *h = new hora_index();
  h->kind = kind;
  h->dim = dim;
  h->ld = (uint64_t)round_up((int64_t)dim, 4);
  if (kind == HORA_INDEX_IVFPQ || kind == HORA_INDEX_PQ) {
    hora_ivfpq_params_default(&h->ivf);
    if (kind == HORA_INDEX_IVFPQ && params) h->ivf = *reinterpret_cast<const hora_ivfpq_params *>(params);
    if (kind == HORA_INDEX_PQ) {
      // a flat PQIndex is the IVF machinery with one list centred at zero
      hora_pq_params pq;
      hora_pq_params_default(&pq);
      if (params) pq = *reinterpret_cast<const hora_pq_params *>(params);
      h->ivf.n_sub = pq.n_sub;
      h->ivf.sub_bits = pq.sub_bits;
      h->ivf.train_epoch = pq.train_epoch;
      h->ivf.n_kmeans_center = 1;
      h->ivf.search_n_center = 1;
    }
    const hora_ivfpq_params &p = h->ivf;
    if (dim > 1024) {
      delete h;
      return fail(HORA_ECAP, "IVF-PQ supports dimension <= 1024");
    }
    if (p.n_sub == 0 || p.n_sub > dim) {
      delete h;
      return fail(HORA_EINVAL, "n_sub must be in [1, dim]");
    }
    if (p.sub_bits < 1 || p.sub_bits > 8) {
      delete h;
      return fail(HORA_ECAP, "sub_bits must be in [1, 8] (8-bit codes)");
    }
    if (p.n_kmeans_center == 0 || p.n_kmeans_center > 16384) {
      delete h;
      return fail(HORA_ECAP, "n_kmeans_center must be in [1, 16384]");
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return fail(HORA_ECUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  *out = h;
  return HORA_OK;
}

int hora_index_free(hora_index *h) {
  if (!h) return HORA_OK;
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  delete h;
  return HORA_OK;
}

static int add_rows(hora_index *h, const float *vecs, const uint64_t *ids, uint64_t n) {
  cudaStream_t s = h->stream;
  const bool dev = is_device_ptr(vecs);
  if (!dev && !host_all_finite(vecs, (int64_t)(n * h->dim)))
    return fail(HORA_ENAN, "invalid float element");
  if (h->n + (int64_t)n >= (int64_t)UINT32_MAX) return fail(HORA_ECAP, "more than 2^32-1 items");
  int64_t need = h->n + (int64_t)n;
  if (need > h->cap_rows) {
    int64_t nc = std::max<int64_t>(need, std::max<int64_t>(1024, h->cap_rows * 3 / 2));
    HORA_TRY(h->base.reserve(sizeof(float) * nc * h->ld, s, true));
    HORA_TRY(h->ids.reserve(sizeof(uint64_t) * nc, s, true));
    h->cap_rows = nc;
  }
  float *dst = h->base.as<float>() + h->n * h->ld;
  if (h->ld != h->dim) HORA_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(float) * n * h->ld, s));
  HORA_CUDA_TRY(cudaMemcpy2DAsync(dst, h->ld * 4, vecs, h->dim * 4, h->dim * 4, n,
                                  cudaMemcpyDefault, s));
  if (dev) {
    int rc = check_device_finite(dst, (int64_t)n, h->ld, h->dim, h->ws.tmp, s);
    if (rc) return rc;
  }
  uint64_t *idd = h->ids.as<uint64_t>() + h->n;
  if (ids) {
    HORA_CUDA_TRY(cudaMemcpyAsync(idd, ids, sizeof(uint64_t) * n, cudaMemcpyDefault, s));
  } else {
    std::vector<uint64_t> seq(n);
    for (uint64_t i = 0; i < n; ++i) seq[i] = (uint64_t)h->n + i;
    HORA_CUDA_TRY(cudaMemcpyAsync(idd, seq.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  h->n += (int64_t)n;
  h->norms_valid = false;
  if (h->lowp) h->lowp.reset();
  return HORA_OK;
}

int hora_add(hora_index *h, const float *vecs, const uint64_t *ids, uint64_t n) {
  if (!h) return fail(HORA_EINVAL, "null index");
  if (n == 0) return HORA_OK;
  if (!vecs) return fail(HORA_EINVAL, "null vectors");
  HORA_TRY(check_not_foreign(vecs, "vectors"));
  HORA_TRY(check_not_foreign(ids, "ids"));
  std::lock_guard<std::mutex> g(h->mu);
  return add_rows(h, vecs, ids, n);
}

int hora_build(hora_index *h, int metric) {
  if (!h) return fail(HORA_EINVAL, "null index");
  if (!metric_supported(metric)) return fail(HORA_EMETRIC, "unknown method");
  std::lock_guard<std::mutex> g(h->mu);
  h->metric = metric;
  if (h->kind == HORA_INDEX_BRUTE_FORCE) {
    // BruteForceIndex::build stores the metric (bruteforce_idx.rs:36-39)
    h->built = true;
    if (metric == M_COS) HORA_TRY(ensure_norms(h, h->stream));
    HORA_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return HORA_OK;
  }
  if (h->kind == HORA_INDEX_PQ && metric == M_COS)
    return fail(HORA_EMETRIC, "PQIndex: CosineSimilarity is not supported (NaN in the reference)");
  int rc = ivf_build(h);
  h->built = rc == HORA_OK;
  return rc;
}

int hora_built(const hora_index *h, int *out) {
  if (!h || !out) return fail(HORA_EINVAL, "null argument");
  *out = h->built ? 1 : 0;
  return HORA_OK;
}

int hora_rebuild(hora_index *h, int metric) {
  (void)h;
  (void)metric;
  return fail(HORA_ENOTIMPL, "not implement");  // ann_index.rs:69-71
}

}  // extern "C"

namespace hora {
// One search on a given workspace and stream (no handle lock: the index is
// read-only during searches; the serving slots call this concurrently).
int search_core(hora_index *h, SearchWorkspace &ws, cudaStream_t s, const float *queries,
                uint64_t nq, uint64_t k, uint64_t nprobe, uint64_t *ids_out, float *dist_out,
                float *vecs_out) {
  HORA_TRY(ws.ev_t0.ensure(true));
  HORA_TRY(ws.ev_t1.ensure(true));
  HORA_CUDA_TRY(cudaEventRecord(ws.ev_t0.ev, s));
  int64_t total = (int64_t)(nq * k);
  // the queries' finiteness is checked on the device and read only before
  // the results are written: no host scan of the queries and no host round
  // trip before the search (the search paths sync on their own by then)
  int rc = stage_queries(h, queries, (int64_t)nq, ws, s, /*defer_check=*/true);
  if (rc == HORA_OK) rc = ws.keys2.reserve(sizeof(uint64_t) * total);
  uint64_t *keys = ws.keys2.as<uint64_t>();
  if (rc == HORA_OK) {
    if (h->kind == HORA_INDEX_BRUTE_FORCE)
      rc = bf_search_keys(h, (int64_t)nq, (int)k, ws, keys, s);
    else
      rc = ivf_search_keys(h, (int64_t)nq, (int)k, (int64_t)nprobe, nullptr, ws, keys, s);
  }
  if (ws.status_pending) {
    ws.status_pending = false;
    if (cudaEventSynchronize(ws.ev_status.ev) != cudaSuccess && rc == HORA_OK)
      rc = fail(HORA_ECUDA, "query check");
    else if (rc == HORA_OK && *ws.h_status.as<uint32_t>())
      rc = fail(HORA_ENAN, "invalid float element");
  }
  if (rc == HORA_OK) {
    const bool dev_ids = is_device_ptr(ids_out), dev_dist = is_device_ptr(dist_out);
    uint64_t *ids_d = ids_out;
    float *dist_d = dist_out;
    if (ids_out && !dev_ids) {
      rc = ws.out_ids.reserve(sizeof(uint64_t) * total);
      ids_d = ws.out_ids.as<uint64_t>();
    }
    if (rc == HORA_OK && dist_out && !dev_dist) {
      rc = ws.out_dist.reserve(sizeof(float) * total);
      dist_d = ws.out_dist.as<float>();
    }
    if (rc == HORA_OK) rc = launch_keys_to_results(keys, total, h->ids.as<uint64_t>(), ids_d, dist_d, s);
    if (rc == HORA_OK && ids_out && !dev_ids)
      rc = cudaMemcpyAsync(ids_out, ids_d, sizeof(uint64_t) * total, cudaMemcpyDeviceToHost, s)
               ? fail(HORA_ECUDA, "D2H ids") : HORA_OK;
    if (rc == HORA_OK && dist_out && !dev_dist)
      rc = cudaMemcpyAsync(dist_out, dist_d, sizeof(float) * total, cudaMemcpyDeviceToHost, s)
               ? fail(HORA_ECUDA, "D2H dist") : HORA_OK;
    if (rc == HORA_OK && vecs_out) {
      const bool dev_v = is_device_ptr(vecs_out);
      float *v_d = vecs_out;
      if (!dev_v) {
        rc = ws.rows.reserve(sizeof(float) * total * h->dim);
        v_d = ws.rows.as<float>();
      }
      if (rc == HORA_OK) rc = launch_gather_rows(keys, total, h->base.as<float>(), h->ld, h->dim, v_d, s);
      if (rc == HORA_OK && !dev_v)
        rc = cudaMemcpyAsync(vecs_out, v_d, sizeof(float) * total * h->dim, cudaMemcpyDeviceToHost, s)
                 ? fail(HORA_ECUDA, "D2H vecs") : HORA_OK;
    }
  }
  cudaError_t re = cudaEventRecord(ws.ev_t1.ev, s);
  cudaError_t se = cudaStreamSynchronize(s);
  if (rc == HORA_OK && se != cudaSuccess) rc = fail(HORA_ECUDA, cudaGetErrorString(se));
  float ms = 0;
  if (re == cudaSuccess && cudaEventElapsedTime(&ms, ws.ev_t0.ev, ws.ev_t1.ev) == cudaSuccess)
    h->last_ms = ms;
  // an error left by a launch or a copy that no status above reported
  cudaError_t le = cudaGetLastError();
  if (rc == HORA_OK && re != cudaSuccess) rc = fail(HORA_ECUDA, cudaGetErrorString(re));
  if (rc == HORA_OK && le != cudaSuccess) rc = fail(HORA_ECUDA, cudaGetErrorString(le));
  return rc;
}
}  // namespace hora

extern "C" {

static int search_common(hora_index *h, const float *queries, uint64_t nq, uint64_t k,
                         uint64_t nprobe, uint64_t *ids_out, float *dist_out, float *vecs_out) {
  if (!h) return fail(HORA_EINVAL, "null index");
  if (nq == 0) return HORA_OK;
  if (!queries || (!ids_out && !dist_out && !vecs_out)) return fail(HORA_EINVAL, "null buffer");
  if (k == 0) return fail(HORA_EINVAL, "k must be positive");
  if (k > 4096) return fail(HORA_ECAP, "k must be <= 4096");
  HORA_TRY(check_not_foreign(queries, "queries"));
  HORA_TRY(check_not_foreign(ids_out, "ids_out"));
  HORA_TRY(check_not_foreign(dist_out, "dist_out"));
  HORA_TRY(check_not_foreign(vecs_out, "vecs_out"));
  std::lock_guard<std::mutex> g(h->mu);
  if (!h->built || h->metric == M_UNKNOWN) return fail(HORA_ENOTBUILT, "unknown method");
  return search_core(h, h->ws, h->stream, queries, nq, k, nprobe, ids_out, dist_out, vecs_out);
}

int hora_search(hora_index *h, const float *queries, uint64_t nq, uint64_t k, uint64_t *ids_out,
                float *dist_out) {
  return search_common(h, queries, nq, k, 0, ids_out, dist_out, nullptr);
}

int hora_search_nprobe(hora_index *h, const float *queries, uint64_t nq, uint64_t k,
                       uint64_t nprobe, uint64_t *ids_out, float *dist_out) {
  return search_common(h, queries, nq, k, nprobe, ids_out, dist_out, nullptr);
}

int hora_search_nodes(hora_index *h, const float *queries, uint64_t nq, uint64_t k,
                      uint64_t *ids_out, float *dist_out, float *vecs_out) {
  return search_common(h, queries, nq, k, 0, ids_out, dist_out, vecs_out);
}

static const char *index_name(int kind) {
  return kind == HORA_INDEX_BRUTE_FORCE ? "BruteForceIndex" : kind == HORA_INDEX_PQ ? "PQIndex" : "IVFPQIndex";
}

int hora_name(const hora_index *h, const char **out) {
  if (!h || !out) return fail(HORA_EINVAL, "null argument");
  *out = index_name(h->kind);
  return HORA_OK;
}

int hora_nodes_size(const hora_index *h, uint64_t *out) {
  if (!h || !out) return fail(HORA_EINVAL, "null argument");
  *out = (uint64_t)h->n;
  return HORA_OK;
}

int hora_dimension(const hora_index *h, uint64_t *out) {
  if (!h || !out) return fail(HORA_EINVAL, "null argument");
  *out = h->dim;
  return HORA_OK;
}

int hora_clear(hora_index *h) {
  if (!h) return fail(HORA_EINVAL, "null index");
  std::lock_guard<std::mutex> g(h->mu);
  cudaStreamSynchronize(h->stream);
  h->n = 0;
  h->built = false;
  h->norms_valid = false;
  h->ivfs.reset();
  h->lowp.reset();
  h->nprobe.reset();
  return HORA_OK;
}

int hora_idx_info(const hora_index *h, char *buf, uint64_t cap) {
  if (!h || !buf || cap == 0) return fail(HORA_EINVAL, "null argument");
  std::string s = "{";
  s += std::string("\"name\":\"") + index_name(h->kind) + "\"";
  s += ",\"dimension\":" + std::to_string(h->dim);
  s += ",\"nodes\":" + std::to_string(h->n);
  s += std::string(",\"metric\":\"") + metric_name(h->metric) + "\"";
  s += std::string(",\"built\":") + (h->built ? "true" : "false");
  s += std::string(",\"precision\":\"") +
       (h->precision == HORA_PREC_FP32 ? "fp32" : h->precision == HORA_PREC_BF16 ? "bf16" : "fp8") + "\"";
  s += ",\"semantics\":{\"Euclidean\":\"squared L2\",\"DotProduct\":\"+<x,q> ascending\","
       "\"CosineSimilarity\":\"-cos(x,q) ascending, 0 for a zero norm\"}";
  s += ",\"device_bytes\":" + std::to_string(h->base.bytes + h->ids.bytes + h->xnorm.bytes +
                                             h->xsq64.bytes + ivf_device_bytes(h));
  s += ",\"last_search_ms\":" + std::to_string(h->last_ms.load());
  s += ",\"last_overflow_rescans\":" + std::to_string(h->last_retries.load());
  s += ",\"last_threshold_probe\":" + std::to_string(h->last_probe.load());
  s += ",\"last_overflow_queries\":" + std::to_string(h->last_overflow_queries.load());
  s += ",\"last_short_lists\":" + std::to_string(h->last_short_lists.load());
  s += ",\"last_fallback_queries\":" + std::to_string(h->last_fallback.load());
  if (h->kind != HORA_INDEX_BRUTE_FORCE) {
    std::string iv;
    ivf_info(h, iv);
    s += ",\"ivfpq\":" + iv;
  }
  s += "}";
  std::snprintf(buf, cap, "%s", s.c_str());
  return s.size() + 1 > cap ? fail(HORA_ECAP, "buffer too small") : HORA_OK;
}

// ---- SerializableIndex --------------------------------------------------------
// File layout (little endian): "HORAGB30", u32 version=1, u32 kind, u64 dim,
// u32 metric, u32 built, u64 n, ivf params (5 x u64), options, n*dim f32
// vectors, n u64 ids, then the IVF-PQ block when kind == IVFPQ.
static const char kMagic[8] = {'H', 'O', 'R', 'A', 'G', 'B', '3', '0'};

int hora_dump(hora_index *h, const char *path) {
  if (!h || !path) return fail(HORA_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(h->mu);
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(HORA_EIO, std::string("unable to write file ") + path);
  uint32_t ver = 1, kind = h->kind, metric = h->metric, built = h->built;
  uint64_t n = h->n;
  bool ok = std::fwrite(kMagic, 8, 1, f) == 1 && std::fwrite(&ver, 4, 1, f) == 1 &&
            std::fwrite(&kind, 4, 1, f) == 1 && std::fwrite(&h->dim, 8, 1, f) == 1 &&
            std::fwrite(&metric, 4, 1, f) == 1 && std::fwrite(&built, 4, 1, f) == 1 &&
            std::fwrite(&n, 8, 1, f) == 1 && std::fwrite(&h->ivf, sizeof(h->ivf), 1, f) == 1;
  int64_t opts[6] = {h->precision, h->rerank, h->cand_cap, h->accum_f64, (int64_t)h->seed,
                     (int64_t)h->train_size};
  ok = ok && std::fwrite(opts, sizeof(opts), 1, f) == 1;
  std::vector<float> rows(n * h->dim);
  std::vector<uint64_t> ids(n);
  if (n) {
    if (cudaMemcpy2D(rows.data(), h->dim * 4, h->base.ptr, h->ld * 4, h->dim * 4, n,
                     cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ids.data(), h->ids.ptr, 8 * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
      std::fclose(f);
      return fail(HORA_ECUDA, "dump: device copy failed");
    }
  }
  ok = ok && (n == 0 || (std::fwrite(rows.data(), 4, rows.size(), f) == rows.size() &&
                         std::fwrite(ids.data(), 8, n, f) == n));
  if (ok && h->kind != HORA_INDEX_BRUTE_FORCE && h->built) ok = ivf_dump(h, f) == HORA_OK;
  std::fclose(f);
  return ok ? HORA_OK : fail(HORA_EIO, std::string("unable to write file ") + path);
}

int hora_load(const char *path, hora_index **out) {
  if (!path || !out) return fail(HORA_EINVAL, "null argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(HORA_EIO, std::string("unable to open file ") + path);
  char magic[8];
  uint32_t ver = 0, kind = 0, metric = 0, built = 0;
  uint64_t dim = 0, n = 0;
  hora_ivfpq_params ivf{};
  int64_t opts[6];
  bool ok = std::fread(magic, 8, 1, f) == 1 && std::memcmp(magic, kMagic, 8) == 0 &&
            std::fread(&ver, 4, 1, f) == 1 && ver == 1 && std::fread(&kind, 4, 1, f) == 1 &&
            std::fread(&dim, 8, 1, f) == 1 && std::fread(&metric, 4, 1, f) == 1 &&
            std::fread(&built, 4, 1, f) == 1 && std::fread(&n, 8, 1, f) == 1 &&
            std::fread(&ivf, sizeof(ivf), 1, f) == 1 && std::fread(opts, sizeof(opts), 1, f) == 1;
  if (!ok || dim == 0 || dim >= (1ull << 20) || n >= UINT32_MAX || kind > HORA_INDEX_PQ) {
    std::fclose(f);
    return fail(HORA_EIO, "corrupt index file");
  }
  hora_index *h = nullptr;
  hora_pq_params pq{ivf.n_sub, ivf.sub_bits, ivf.train_epoch};
  const void *params = kind == HORA_INDEX_IVFPQ ? (const void *)&ivf : kind == HORA_INDEX_PQ ? (const void *)&pq : nullptr;
  int rc = hora_index_create((int)kind, dim, params, &h);
  if (rc) {
    std::fclose(f);
    return rc;
  }
  h->precision = (int)opts[0];
  h->rerank = (int)opts[1];
  h->cand_cap = (int)opts[2];
  h->accum_f64 = (int)opts[3];
  h->seed = (uint64_t)opts[4];
  h->train_size = (uint64_t)opts[5];
  std::vector<float> rows(n * dim);
  std::vector<uint64_t> ids(n);
  ok = n == 0 || (std::fread(rows.data(), 4, rows.size(), f) == rows.size() &&
                  std::fread(ids.data(), 8, n, f) == n);
  if (ok && n) rc = add_rows(h, rows.data(), ids.data(), n);
  if (!ok || rc) {
    std::fclose(f);
    hora_index_free(h);
    return rc ? rc : fail(HORA_EIO, "corrupt index file");
  }
  h->metric = (int)metric;
  if (kind != HORA_INDEX_BRUTE_FORCE && built) {
    rc = ivf_load(h, f);
    if (rc) {
      std::fclose(f);
      hora_index_free(h);
      return rc;
    }
  }
  std::fclose(f);
  h->built = built != 0;
  if (h->built && metric == M_COS) ensure_norms(h, h->stream);
  cudaStreamSynchronize(h->stream);
  *out = h;
  return HORA_OK;
}

// ---- options --------------------------------------------------------------------
int hora_set_option(hora_index *h, int key, double v) {
  if (!h) return fail(HORA_EINVAL, "null index");
  std::lock_guard<std::mutex> g(h->mu);
  switch (key) {
    case HORA_OPT_PRECISION:
      if (v != HORA_PREC_FP32 && v != HORA_PREC_BF16 && v != HORA_PREC_FP8)
        return fail(HORA_EINVAL, "precision must be 0 (fp32), 1 (bf16) or 2 (fp8)");
      h->precision = (int)v;
      return HORA_OK;
    case HORA_OPT_RERANK:
      if (v < 0 || v > 16384) return fail(HORA_ECAP, "rerank must be in [0, 16384]");
      h->rerank = (int)v;
      return HORA_OK;
    case HORA_OPT_SEED: h->seed = (uint64_t)v; return HORA_OK;
    case HORA_OPT_TRAIN_SIZE: h->train_size = (uint64_t)(v < 0 ? 0 : v); return HORA_OK;
    case HORA_OPT_ACCUM_F64: h->accum_f64 = v != 0; return HORA_OK;
    case HORA_OPT_CAND_CAP:
      if (v < 256 || v > 16384) return fail(HORA_ECAP, "candidate capacity must be in [256, 16384]");
      h->cand_cap = (int)v;
      return HORA_OK;
    case HORA_OPT_LEARNED_NPROBE: h->learned_nprobe = v != 0; return HORA_OK;
    case HORA_OPT_NPROBE_MARGIN: h->nprobe_margin = v; return HORA_OK;
    case HORA_OPT_NPROBE_MAX: h->nprobe_max = (int)(v < 0 ? 0 : v); return HORA_OK;
    case HORA_OPT_NPROBE_PHASE1:
      if (v < 0 || v > 64) return fail(HORA_ECAP, "phase-1 probes must be in [0, 64]");
      h->nprobe_phase1 = (int)v;
      return HORA_OK;
    case HORA_OPT_IVF_RERANK:
      if (v < 0 || v > 4096) return fail(HORA_ECAP, "ivf rerank must be in [0, 4096]");
      h->ivf_rerank = (int)v;
      return HORA_OK;
    case HORA_OPT_BF_PROBE: h->bf_probe = v != 0; return HORA_OK;
    case HORA_OPT_EXACT_TC: h->exact_tc = v != 0; return HORA_OK;
  }
  return fail(HORA_EINVAL, "unknown option");
}

int hora_get_option(const hora_index *h, int key, double *out) {
  if (!h || !out) return fail(HORA_EINVAL, "null argument");
  switch (key) {
    case HORA_OPT_PRECISION: *out = h->precision; return HORA_OK;
    case HORA_OPT_RERANK: *out = h->rerank; return HORA_OK;
    case HORA_OPT_SEED: *out = (double)h->seed; return HORA_OK;
    case HORA_OPT_TRAIN_SIZE: *out = (double)h->train_size; return HORA_OK;
    case HORA_OPT_ACCUM_F64: *out = h->accum_f64; return HORA_OK;
    case HORA_OPT_CAND_CAP: *out = h->cand_cap; return HORA_OK;
    case HORA_OPT_LEARNED_NPROBE: *out = h->learned_nprobe; return HORA_OK;
    case HORA_OPT_NPROBE_MARGIN: *out = h->nprobe_margin; return HORA_OK;
    case HORA_OPT_NPROBE_MAX: *out = h->nprobe_max; return HORA_OK;
    case HORA_OPT_IVF_RERANK: *out = h->ivf_rerank; return HORA_OK;
    case HORA_OPT_NPROBE_PHASE1: *out = h->nprobe_phase1; return HORA_OK;
    case HORA_OPT_BF_PROBE: *out = h->bf_probe; return HORA_OK;
    case HORA_OPT_EXACT_TC: *out = h->exact_tc; return HORA_OK;
  }
  return fail(HORA_EINVAL, "unknown option");
}

int hora_ivfpq_layout(const hora_index *h, uint64_t *n_list, uint64_t *n_sub, uint64_t *sub_bits,
                      uint64_t *dmax) {
  if (!h) return fail(HORA_EINVAL, "null index");
  return ivf_layout(h, n_list, n_sub, sub_bits, dmax);
}

int hora_ivfpq_export(const hora_index *h, float *centers, int64_t *offsets, int64_t *items,
                      float *codebooks, uint8_t *codes, uint8_t *trained) {
  if (!h) return fail(HORA_EINVAL, "null index");
  return ivf_export(h, centers, offsets, items, codebooks, codes, trained);
}

int hora_ivfpq_set_codebooks(hora_index *h, const float *centers, const float *codebooks) {
  if (!h || !centers || !codebooks) return fail(HORA_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(h->mu);
  return ivf_set_codebooks(h, centers, codebooks);
}

}  // extern "C"
