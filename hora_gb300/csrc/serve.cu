// serve.cu — continuous-batching request loop (no reference counterpart: the
// reference serves one query per call, src/core/ann_index.rs:91-97).
//
// Requests (any batch size, any k, any of the server's indexes) are queued
// from any thread.  Each of n_slots workers owns a CUDA stream and a search
// workspace.  A free worker takes the oldest request whose working-set bytes
// fit under the HBM budget next to the requests already in flight, and folds
// in every further queued request for the same index whose k gives the same
// candidate width (search_width: any k on the exact paths; every k up to the
// rerank width on the approximate ones) and that still fits (up to 8,192
// queries per batch); the batch runs at its largest k and each request takes
// its first k columns.  Requests arriving while others run join the next
// batch on the next free slot.  Work on different slots
// overlaps on the GPU.  Results are bit-identical to running each request
// alone: every path is deterministic per query and a batch only concatenates
// queries.  Latency is measured per request from submit to completion.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>
#include <vector>

#include "index.h"

namespace hora {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  uint32_t index_no = 0;
  const float *q = nullptr;
  uint64_t nq = 0, k = 0;
  uint64_t *ids = nullptr;
  float *dist = nullptr;
  size_t bytes = 0;
  Clock::time_point t_submit, t_done;
  int status = HORA_OK;
  std::string error;
  bool done = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  SearchWorkspace ws;
  float *h_q = nullptr;
  uint64_t *h_ids = nullptr;
  float *h_dist = nullptr;
  size_t cap_q = 0, cap_r = 0;
  std::thread th;
};

}  // namespace hora

struct hora_server {
  std::vector<hora_index *> idx;
  uint64_t budget = 0;
  uint64_t admitted = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<hora::Request *> queue;
  std::unordered_map<uint64_t, hora::Request *> all;
  std::vector<std::unique_ptr<hora::Slot>> slots;
  bool stop = false;
  uint64_t next_ticket = 1;
  int device = 0;
  // statistics
  std::vector<double> lat_ms;
  uint64_t completed = 0, completed_q = 0, rejected = 0, inflight = 0, max_inflight = 0;
  uint64_t max_admitted = 0;
  uint64_t batches = 0, mixed_k_batches = 0;
};

namespace hora {

constexpr uint64_t kMaxBatchQueries = 8192;

// Device working set of one request of nq queries (or of a batch at the
// batch's largest k): staged queries and their copies, k-best and candidate
// lists, outputs, and the per-search buffers with minimum sizes (the
// probed threshold buffers are sized for at least 1,024 queries, the IVF
// pair tables per list) — an upper estimate of what its search reserves in
// the slot's workspace.
static size_t request_bytes(const hora_index *h, uint64_t nq, uint64_t k) {
  const size_t ld = h->ld, Dp = (size_t)round_up((int64_t)h->dim, 64) * 2;  // BF16 row, or 128 FP8 bytes
  size_t per_q = ld * 4 * 2 + 64 + k * (8 + 8 + 8 + 12);  // queries (and a gathered copy), norms, keys, outputs
  size_t fixed = 64 << 10;                                  // small buffers and 256-byte minimums
  if (h->kind == HORA_INDEX_BRUTE_FORCE) {
    const int R = std::max<int>((int)k, lowp_rerank_width(h, (int)k));
    const size_t cap = (size_t)round_up(std::max(h->cand_cap, 2 * R), 128);
    per_q += Dp * 2 + cap * 8 + (size_t)R * 16 + 64;
    // starting thresholds: per query (a power of two >= 1,024 of them) the
    // pivot key, bucket slot, member keys, threshold, position, query copy
    // and share of a work item (4,096 pivots at most), and the bucketing's
    // per-block pivot counts (a block per 128 queries at most); for wide
    // lists the sample pass's list and candidates (at most 180 + 2,048 keys)
    const size_t nres = std::max<size_t>(1024, nq);
    fixed += 2 * nres * (8 + 4 + 1024 * 4 + 4 + 4 + Dp + 1) + (size_t)4097 * 48 +
             (2 * nres / 128 + 1) * (size_t)4097 * 4;
    if (lowp_probe_kind(h, R) == 2) per_q += 8 * (180 + 2048 + 32) + 8;
  } else {
    const size_t C = h->ivf.n_kmeans_center;
    size_t pmax = std::max<size_t>(32, std::max<size_t>(h->ivf.search_n_center, (size_t)h->nprobe_max));
    pmax = std::min(pmax, C);
    const size_t R = std::max<size_t>(k, (size_t)h->ivf_rerank);
    per_q += C * 4 + pmax * (8 + 12 + 4) + pmax * R * 8 + R * 16 + 40 * 4 + 16;
    // the certified coarse probe: the rescored centres and their count, the
    // BF16 query copy, its f32 squared norm and slack
    if (coarse_tc_eligible(h)) per_q += C * 8 + 4 + Dp + 8;
    fixed += (C + 1) * 32 + C * 4;
  }
  return per_q * nq + fixed;
}

// The candidates a search of index h keeps before its final k best: 0 when
// the k best are a prefix of any larger k's (every exact path, and IVF-PQ
// without a rerank, whose per-list k best contain the global k best).  Two
// requests with the same width run as one batch at the larger k, each
// taking the first k of its rows: the same result as alone.
static int64_t search_width(const hora_index *h, uint64_t k) {
  if (h->kind == HORA_INDEX_BRUTE_FORCE) return h->precision == HORA_PREC_FP32 ? 0 : lowp_rerank_width(h, (int)k);
  if (h->ivf_rerank <= 0) return 0;
  return ivf_rerank_width(h, (int)k);
}

static int ensure_pinned(Slot &sl, size_t nq, size_t dim, size_t kk) {
  if (nq * dim > sl.cap_q) {
    if (sl.h_q) cudaFreeHost(sl.h_q);
    sl.cap_q = std::max(nq * dim, sl.cap_q * 2);
    HORA_CUDA_TRY(cudaHostAlloc(&sl.h_q, sl.cap_q * 4, cudaHostAllocDefault));
  }
  if (nq * kk > sl.cap_r) {
    if (sl.h_ids) cudaFreeHost(sl.h_ids);
    if (sl.h_dist) cudaFreeHost(sl.h_dist);
    sl.cap_r = std::max(nq * kk, sl.cap_r * 2);
    HORA_CUDA_TRY(cudaHostAlloc(&sl.h_ids, sl.cap_r * 8, cudaHostAllocDefault));
    HORA_CUDA_TRY(cudaHostAlloc(&sl.h_dist, sl.cap_r * 4, cudaHostAllocDefault));
  }
  return HORA_OK;
}

static void worker(hora_server *sv, int slot_no) {
  cudaSetDevice(sv->device);
  Slot &sl = *sv->slots[slot_no];
  std::vector<Request *> batch;
  for (;;) {
    batch.clear();
    {
      std::unique_lock<std::mutex> g(sv->mu);
      sv->cv_work.wait(g, [&] {
        if (sv->stop) return true;
        if (sv->queue.empty()) return false;
        return sv->admitted + sv->queue.front()->bytes <= sv->budget;
      });
      if (sv->stop && sv->queue.empty()) return;
      if (sv->queue.empty() || sv->admitted + sv->queue.front()->bytes > sv->budget) continue;
      Request *head = sv->queue.front();
      sv->queue.pop_front();
      batch.push_back(head);
      sv->admitted += head->bytes;
      uint64_t total = head->nq, kmax = head->k;
      const hora_index *hi = sv->idx[head->index_no];
      const int64_t width = search_width(hi, head->k);
      for (auto it = sv->queue.begin(); it != sv->queue.end();) {
        Request *r = *it;
        if (r->index_no != head->index_no || search_width(hi, r->k) != width || total + r->nq > kMaxBatchQueries) {
          ++it;
          continue;
        }
        // the batch runs at its largest k: every member is charged at it
        const uint64_t kn = std::max(kmax, r->k);
        size_t extra = request_bytes(hi, r->nq, kn);
        if (kn > kmax)
          for (Request *m : batch) extra += request_bytes(hi, m->nq, kn) - m->bytes;
        if (sv->admitted + extra > sv->budget) {
          ++it;
          continue;
        }
        if (kn > kmax)
          for (Request *m : batch) m->bytes = request_bytes(hi, m->nq, kn);
        r->bytes = request_bytes(hi, r->nq, kn);
        sv->admitted += extra;
        kmax = kn;
        batch.push_back(r);
        total += r->nq;
        it = sv->queue.erase(it);
      }
      sv->batches += 1;
      for (Request *m : batch)
        if (m->k != kmax) {
          sv->mixed_k_batches += 1;
          break;
        }
      sv->inflight += batch.size();
      sv->max_inflight = std::max(sv->max_inflight, sv->inflight);
      sv->max_admitted = std::max(sv->max_admitted, sv->admitted);
    }
    // run the batch at its largest k
    hora_index *h = sv->idx[batch[0]->index_no];
    const uint64_t dim = h->dim;
    uint64_t total = 0, k = 0;
    for (Request *r : batch) {
      total += r->nq;
      k = std::max(k, r->k);
    }
    int rc = ensure_pinned(sl, total, dim, k);
    std::string err;
    if (rc == HORA_OK) {
      uint64_t off = 0;
      for (Request *r : batch) {
        std::memcpy(sl.h_q + off * dim, r->q, sizeof(float) * r->nq * dim);
        off += r->nq;
      }
      rc = search_core(h, sl.ws, sl.stream, sl.h_q, total, k, 0, sl.h_ids, sl.h_dist, nullptr);
      if (rc == HORA_OK) {
        off = 0;
        for (Request *r : batch) {
          // each request's first r->k of the batch's k columns
          for (uint64_t i = 0; i < r->nq; ++i) {
            std::memcpy(r->ids + i * r->k, sl.h_ids + (off + i) * k, sizeof(uint64_t) * r->k);
            std::memcpy(r->dist + i * r->k, sl.h_dist + (off + i) * k, sizeof(float) * r->k);
          }
          off += r->nq;
        }
      }
    }
    if (rc != HORA_OK) err = hora_last_error();
    const auto now = Clock::now();
    {
      std::lock_guard<std::mutex> g(sv->mu);
      for (Request *r : batch) {
        r->status = rc;
        r->error = err;
        r->t_done = now;
        r->done = true;
        sv->admitted -= r->bytes;
        sv->inflight -= 1;
        if (rc == HORA_OK) {
          sv->completed += 1;
          sv->completed_q += r->nq;
          sv->lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
        }
      }
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
}

}  // namespace hora

using namespace hora;

extern "C" {

int hora_server_create(hora_index *const *indexes, uint32_t n_indexes, uint32_t n_slots,
                       uint64_t hbm_budget_bytes, hora_server **out) {
  if (!indexes || !n_indexes || !out) return fail(HORA_EINVAL, "null argument");
  if (n_slots == 0 || n_slots > 64) return fail(HORA_ECAP, "n_slots must be in [1, 64]");
  *out = nullptr;
  for (uint32_t i = 0; i < n_indexes; ++i) {
    if (!indexes[i]) return fail(HORA_EINVAL, "null index");
    HORA_TRY(prepare_for_concurrent_search(indexes[i]));
  }
  hora_server *sv = new hora_server();
  sv->idx.assign(indexes, indexes + n_indexes);
  sv->budget = hbm_budget_bytes ? hbm_budget_bytes : UINT64_MAX;
  cudaGetDevice(&sv->device);
  for (uint32_t i = 0; i < n_slots; ++i) sv->slots.emplace_back(new Slot());
  for (uint32_t i = 0; i < n_slots; ++i) {
    if (cudaStreamCreateWithFlags(&sv->slots[i]->stream, cudaStreamNonBlocking) != cudaSuccess) {
      for (uint32_t j = 0; j < i; ++j) cudaStreamDestroy(sv->slots[j]->stream);
      delete sv;
      return fail(HORA_ECUDA, "cudaStreamCreate failed");
    }
  }
  for (uint32_t i = 0; i < n_slots; ++i) sv->slots[i]->th = std::thread(worker, sv, (int)i);
  *out = sv;
  return HORA_OK;
}

int hora_server_free(hora_server *sv) {
  if (!sv) return HORA_OK;
  {
    std::lock_guard<std::mutex> g(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto &slp : sv->slots)
    if (slp->th.joinable()) slp->th.join();
  for (auto &slp : sv->slots) {
    hora::Slot &sl = *slp;
    cudaStreamSynchronize(sl.stream);
    cudaStreamDestroy(sl.stream);
    if (sl.h_q) cudaFreeHost(sl.h_q);
    if (sl.h_ids) cudaFreeHost(sl.h_ids);
    if (sl.h_dist) cudaFreeHost(sl.h_dist);
  }
  for (auto &kv : sv->all) delete kv.second;
  for (Request *r : sv->queue) (void)r;  // owned by `all`
  delete sv;
  return HORA_OK;
}

int hora_server_submit(hora_server *sv, uint32_t index_no, const float *queries, uint64_t nq,
                       uint64_t k, uint64_t *ids_out, float *dist_out, uint64_t *ticket) {
  if (!sv || !queries || !ids_out || !dist_out || !ticket) return fail(HORA_EINVAL, "null argument");
  if (index_no >= sv->idx.size()) return fail(HORA_EINVAL, "index_no out of range");
  if (nq == 0 || k == 0) return fail(HORA_EINVAL, "empty request");
  if (nq > kMaxBatchQueries) return fail(HORA_ECAP, "at most 8192 queries per request");
  if (k > 1024) return fail(HORA_ECAP, "k must be <= 1024");
  Request *r = new Request();
  r->index_no = index_no;
  r->q = queries;
  r->nq = nq;
  r->k = k;
  r->ids = ids_out;
  r->dist = dist_out;
  r->bytes = request_bytes(sv->idx[index_no], nq, k);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(sv->mu);
    if (r->bytes > sv->budget) {
      sv->rejected += 1;
      delete r;
      return fail(HORA_EOOM, "request exceeds the HBM budget");
    }
    r->ticket = sv->next_ticket++;
    sv->all[r->ticket] = r;
    sv->queue.push_back(r);
    *ticket = r->ticket;
  }
  sv->cv_work.notify_one();
  return HORA_OK;
}

int hora_server_wait(hora_server *sv, uint64_t ticket, int64_t timeout_ms, double *latency_ms) {
  if (!sv) return fail(HORA_EINVAL, "null server");
  std::unique_lock<std::mutex> g(sv->mu);
  auto it = sv->all.find(ticket);
  if (it == sv->all.end()) return fail(HORA_EINVAL, "unknown ticket");
  Request *r = it->second;
  auto pred = [&] { return r->done; };
  if (timeout_ms < 0) {
    sv->cv_done.wait(g, pred);
  } else if (!sv->cv_done.wait_for(g, std::chrono::milliseconds(timeout_ms), pred)) {
    return fail(HORA_ETIMEDOUT, "request not finished");
  }
  int rc = r->status;
  std::string err = r->error;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  sv->all.erase(it);
  delete r;
  return rc == HORA_OK ? HORA_OK : fail(rc, err);
}

int hora_server_request_bytes(hora_server *sv, uint32_t index_no, uint64_t nq, uint64_t k, uint64_t *out) {
  if (!sv || !out) return fail(HORA_EINVAL, "null argument");
  if (index_no >= sv->idx.size()) return fail(HORA_EINVAL, "index_no out of range");
  *out = request_bytes(sv->idx[index_no], nq, k);
  return HORA_OK;
}

int hora_server_info(hora_server *sv, char *buf, uint64_t cap) {
  if (!sv || !buf || cap == 0) return fail(HORA_EINVAL, "null argument");
  std::string s;
  {
    std::lock_guard<std::mutex> g(sv->mu);
    s = "{\"batches\":" + std::to_string(sv->batches) + ",\"mixed_k_batches\":" +
        std::to_string(sv->mixed_k_batches) + ",\"slot_workspace_bytes\":[";
    for (size_t i = 0; i < sv->slots.size(); ++i)
      s += (i ? "," : "") + std::to_string(sv->slots[i]->ws.device_bytes());
    s += "]}";
  }
  std::snprintf(buf, cap, "%s", s.c_str());
  return s.size() + 1 > cap ? fail(HORA_ECAP, "buffer too small") : HORA_OK;
}

int hora_server_stats(hora_server *sv, double *out) {
  if (!sv || !out) return fail(HORA_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(sv->mu);
  std::vector<double> l = sv->lat_ms;
  double p50 = 0, p99 = 0;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    p50 = l[(size_t)(0.50 * (l.size() - 1))];
    p99 = l[(size_t)(0.99 * (l.size() - 1))];
  }
  out[0] = (double)sv->completed;
  out[1] = (double)sv->completed_q;
  out[2] = p50;
  out[3] = p99;
  out[4] = (double)sv->max_inflight;
  out[5] = (double)sv->max_admitted;
  out[6] = (double)sv->rejected;
  return HORA_OK;
}

}  // extern "C"
