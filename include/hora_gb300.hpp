// hora_gb300.hpp — C++ mirror of hora's index API over the C ABI
// (include/hora_gb300.h).  Header only.
//
// The reference's interface is trait ANNIndex<E, T> (src/core/ann_index.rs:
// 25-121) plus SerializableIndex (:141-158), implemented by BruteForceIndex
// (src/index/bruteforce_idx.rs) and IVFPQIndex (src/index/pq_idx.rs).  This
// header restores that shape in C++: E is float, T is any copyable id type
// (mapped to the library's uint64 row ids through a table kept here, as the
// reference keeps an Option<T> per Node), Result<_, &'static str> becomes
// hora::Result, and the provided methods (add, madd, search, search_nodes)
// are implemented on top of the batched C calls.
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "hora_gb300.h"

namespace hora {

// Metric (src/core/metrics.rs:5-13), same variant order.
enum class Metric : int {
  Unknown = HORA_METRIC_UNKNOWN,
  Manhattan = HORA_METRIC_MANHATTAN,
  DotProduct = HORA_METRIC_DOT_PRODUCT,
  Euclidean = HORA_METRIC_EUCLIDEAN,
  CosineSimilarity = HORA_METRIC_COSINE_SIMILARITY,
  Angular = HORA_METRIC_ANGULAR,
};

// Result<(), &'static str>: ok() or the library's error message.
struct Result {
  int code = HORA_OK;
  std::string error;
  bool ok() const { return code == HORA_OK; }
  static Result from(int rc) {
    Result r;
    r.code = rc;
    if (rc != HORA_OK) r.error = hora_last_error();
    return r;
  }
};

// Node<E, T> (src/core/node.rs:93-97).
template <class T>
struct Node {
  std::vector<float> vectors;
  bool has_idx = false;
  T idx{};
};

// BruteForceParams {} (src/index/bruteforce_params.rs:5-14).
struct BruteForceParams {};

// IVFPQParams with the reference's defaults (src/index/pq_params.rs:80-91)
// and builder setters (:52-78).
struct IVFPQParams {
  hora_ivfpq_params p;
  IVFPQParams() { hora_ivfpq_params_default(&p); }
  IVFPQParams &n_sub(uint64_t v) { p.n_sub = v; return *this; }
  IVFPQParams &sub_bits(uint64_t v) { p.sub_bits = v; return *this; }
  IVFPQParams &n_kmeans_center(uint64_t v) { p.n_kmeans_center = v; return *this; }
  IVFPQParams &search_n_center(uint64_t v) { p.search_n_center = v; return *this; }
  IVFPQParams &train_epoch(uint64_t v) { p.train_epoch = v; return *this; }
};

// PQParams (src/index/pq_params.rs:8-41), same builder style.
struct PQParams {
  hora_pq_params p;
  PQParams() { hora_pq_params_default(&p); }
  PQParams &n_sub(uint64_t v) { p.n_sub = v; return *this; }
  PQParams &sub_bits(uint64_t v) { p.sub_bits = v; return *this; }
  PQParams &train_epoch(uint64_t v) { p.train_epoch = v; return *this; }
};

// ANNIndex<f32, T> for one library handle.
template <class T>
class ANNIndex {
 public:
  ANNIndex(const ANNIndex &) = delete;
  ANNIndex &operator=(const ANNIndex &) = delete;
  ANNIndex(ANNIndex &&o) noexcept : h_(o.h_), dim_(o.dim_), ids_(std::move(o.ids_)) { o.h_ = nullptr; }
  virtual ~ANNIndex() { hora_index_free(h_); }

  // build (ann_index.rs:30)
  Result build(Metric mt) { return Result::from(hora_build(h_, (int)mt)); }
  // add_node (ann_index.rs:36)
  Result add_node(const Node<T> &n) { return add(n.vectors.data(), n.idx); }
  // add (ann_index.rs:41-43)
  Result add(const float *vs, const T &idx) { return madd(vs, &idx, 1); }
  Result add(const std::vector<float> &vs, const T &idx) {
    if (vs.size() != dim_) return Result{HORA_EDIM, "dimension is different"};
    return add(vs.data(), idx);
  }
  // madd (ann_index.rs:48-59): n row-major vectors and their ids
  Result madd(const float *vss, const T *indices, uint64_t n) {
    std::vector<uint64_t> rows(n);
    for (uint64_t i = 0; i < n; ++i) rows[i] = ids_.size() + i;
    Result r = Result::from(hora_add(h_, vss, rows.data(), n));
    if (r.ok()) ids_.insert(ids_.end(), indices, indices + n);
    return r;
  }
  // built (ann_index.rs:64)
  bool built() const {
    int b = 0;
    hora_built(h_, &b);
    return b != 0;
  }
  // rebuild (ann_index.rs:69-71): "not implement"
  Result rebuild(Metric mt) { return Result::from(hora_rebuild(h_, (int)mt)); }

  // Batched search: nq row-major queries; per query the ids ascending.
  Result search_batch(const float *queries, uint64_t nq, uint64_t k, std::vector<std::vector<T>> &out,
                      std::vector<std::vector<float>> *dist = nullptr) {
    std::vector<uint64_t> rows(nq * k);
    std::vector<float> d(nq * k);
    Result r = Result::from(hora_search(h_, queries, nq, k, rows.data(), d.data()));
    if (!r.ok()) return r;
    out.assign(nq, {});
    if (dist) dist->assign(nq, {});
    for (uint64_t q = 0; q < nq; ++q)
      for (uint64_t j = 0; j < k; ++j) {
        uint64_t row = rows[q * k + j];
        if (row == HORA_NO_ID) break;
        out[q].push_back(ids_[row]);
        if (dist) (*dist)[q].push_back(d[q * k + j]);
      }
    return r;
  }
  // search (ann_index.rs:91-97)
  std::vector<T> search(const std::vector<float> &item, uint64_t k) {
    std::vector<std::vector<T>> out;
    if (item.size() != dim_ || !search_batch(item.data(), 1, k, out).ok()) return {};
    return out[0];
  }
  // search_nodes (ann_index.rs:81-84)
  std::vector<std::pair<Node<T>, float>> search_nodes(const std::vector<float> &item, uint64_t k) {
    std::vector<uint64_t> rows(k);
    std::vector<float> d(k), v(k * dim_);
    std::vector<std::pair<Node<T>, float>> res;
    if (item.size() != dim_ ||
        hora_search_nodes(h_, item.data(), 1, k, rows.data(), d.data(), v.data()) != HORA_OK)
      return res;
    for (uint64_t j = 0; j < k && rows[j] != HORA_NO_ID; ++j) {
      Node<T> n;
      n.vectors.assign(v.begin() + j * dim_, v.begin() + (j + 1) * dim_);
      n.has_idx = true;
      n.idx = ids_[rows[j]];
      res.emplace_back(std::move(n), d[j]);
    }
    return res;
  }

  const char *name() const {
    const char *s = "";
    hora_name(h_, &s);
    return s;
  }
  uint64_t nodes_size() const { return ids_.size(); }
  uint64_t dimension() const { return dim_; }
  void clear() {
    hora_clear(h_);
    ids_.clear();
  }
  std::string idx_info() const {
    std::string buf(1 << 16, '\0');
    if (hora_idx_info(h_, &buf[0], buf.size()) != HORA_OK) return "not implement";
    buf.resize(std::char_traits<char>::length(buf.c_str()));
    return buf;
  }
  Result set_option(hora_option key, double value) { return Result::from(hora_set_option(h_, key, value)); }
  hora_index *handle() const { return h_; }

 protected:
  ANNIndex(int kind, uint64_t dim, const void *params) : dim_(dim) {
    if (hora_index_create(kind, dim, params, &h_) != HORA_OK) h_ = nullptr;
  }
  hora_index *h_ = nullptr;
  uint64_t dim_ = 0;
  std::vector<T> ids_;
};

// BruteForceIndex<f32, T> (src/index/bruteforce_idx.rs:24-30)
template <class T>
class BruteForceIndex : public ANNIndex<T> {
 public:
  BruteForceIndex(uint64_t dimension, const BruteForceParams & = {})
      : ANNIndex<T>(HORA_INDEX_BRUTE_FORCE, dimension, nullptr) {}
};

// IVFPQIndex<f32, T> (src/index/pq_idx.rs:294-330), a.k.a. PQIVFIndex
template <class T>
class IVFPQIndex : public ANNIndex<T> {
 public:
  IVFPQIndex(uint64_t dimension, const IVFPQParams &params = {})
      : ANNIndex<T>(HORA_INDEX_IVFPQ, dimension, &params.p) {}
};
template <class T>
using PQIVFIndex = IVFPQIndex<T>;

// PQIndex<f32, T> (src/index/pq_idx.rs:21-265): the flat product-quantized index.
template <class T>
class PQIndex : public ANNIndex<T> {
 public:
  PQIndex(uint64_t dimension, const PQParams &params = {})
      : ANNIndex<T>(HORA_INDEX_PQ, dimension, &params.p) {}
};

}  // namespace hora
