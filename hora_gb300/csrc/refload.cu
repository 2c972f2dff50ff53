// refload.cu — SerializableIndex::load for files the reference itself wrote.
//
// The reference dumps its index structs with bincode 1.3's default encoding
// (src/index/bruteforce_idx.rs:84-106, pq_idx.rs:243-265, 488-523):
// little-endian fixed-width integers, usize as u64, Vec<T> as a u64 length
// and the elements, Option<T> as a u8 tag (0 None, 1 Some) and the value,
// bool as a u8, Box<T> as T, a unit enum variant (Metric) as its u32 index,
// struct fields in declaration order.  Element type f32, id type usize (the
// reference's bindings).  The parsed index is rebuilt through the library's
// own paths: vectors and ids are added, and a trained PQ / IVF-PQ index
// gets the file's coarse centres and codebooks (lists and codes are
// recomputed on the GPU, bit-exact given identical codebooks, and the lists
// are checked against the file's inverted lists).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "index.h"

using namespace hora;

namespace {

struct Reader {
  std::vector<uint8_t> buf;
  size_t at = 0;
  bool ok = true;

  bool need(size_t n) {
    if (!ok || buf.size() - at < n) ok = false;
    return ok;
  }
  uint64_t u64() {
    uint64_t v = 0;
    if (need(8)) std::memcpy(&v, buf.data() + at, 8), at += 8;
    return v;
  }
  uint32_t u32() {
    uint32_t v = 0;
    if (need(4)) std::memcpy(&v, buf.data() + at, 4), at += 4;
    return v;
  }
  uint8_t u8() {
    uint8_t v = 0;
    if (need(1)) v = buf[at++];
    return v;
  }
  // a length that must fit in what is left, counting `unit` bytes per element
  uint64_t len(size_t unit) {
    const uint64_t n = u64();
    if (ok && unit && n > (buf.size() - at) / unit) ok = false;
    return ok ? n : 0;
  }
  std::vector<float> f32s() {
    const uint64_t n = len(4);
    std::vector<float> v(n);
    if (n && need(4 * n)) std::memcpy(v.data(), buf.data() + at, 4 * n), at += 4 * n;
    return v;
  }
  std::vector<uint64_t> u64s() {
    const uint64_t n = len(8);
    std::vector<uint64_t> v(n);
    if (n && need(8 * n)) std::memcpy(v.data(), buf.data() + at, 8 * n), at += 8 * n;
    return v;
  }
  std::vector<std::vector<uint64_t>> u64s2() {
    const uint64_t n = len(8);
    std::vector<std::vector<uint64_t>> v;
    for (uint64_t i = 0; ok && i < n; ++i) v.push_back(u64s());
    return v;
  }
  std::vector<std::vector<float>> f32s2() {
    const uint64_t n = len(8);
    std::vector<std::vector<float>> v;
    for (uint64_t i = 0; ok && i < n; ++i) v.push_back(f32s());
    return v;
  }
};

// Vec<Node<f32, usize>> (node.rs:93-97): rows appended to `rows` (dim each),
// ids to `ids` (a missing id becomes the row number, as hora_add does).
struct Nodes {
  std::vector<float> rows;
  std::vector<uint64_t> ids;
  uint64_t dim = 0, n = 0;
};

bool read_nodes(Reader &r, Nodes &out) {
  const uint64_t n = r.len(9);  // at least a length and a tag per node
  for (uint64_t i = 0; r.ok && i < n; ++i) {
    std::vector<float> v = r.f32s();
    const uint8_t tag = r.u8();
    const uint64_t id = tag == 1 ? r.u64() : out.n;
    if (tag > 1) r.ok = false;
    if (!r.ok) break;
    if (out.n == 0 && out.rows.empty()) out.dim = v.size();
    if (v.size() != out.dim) {
      r.ok = false;
      break;
    }
    out.rows.insert(out.rows.end(), v.begin(), v.end());
    out.ids.push_back(id);
    ++out.n;
  }
  return r.ok;
}

// PQIndex<f32, usize> fields in declaration order (pq_idx.rs:21-43).
struct RefPQ {
  uint64_t dimension = 0, n_sub = 0, sub_dimension = 0, sub_bits = 0, train_epoch = 0;
  std::vector<std::vector<std::vector<float>>> centers;  // [n_sub][K][len]
  bool is_trained = false;
  Nodes nodes;
  uint32_t mt = 0;
};

bool read_pq(Reader &r, RefPQ &p) {
  p.dimension = r.u64();
  p.n_sub = r.u64();
  p.sub_dimension = r.u64();
  (void)r.u64s2();  // _dimension_range
  p.sub_bits = r.u64();
  (void)r.u64();  // _sub_bytes
  (void)r.u64();  // _n_sub_center
  (void)r.u64();  // _code_bytes
  p.train_epoch = r.u64();
  const uint64_t m = r.len(8);
  for (uint64_t i = 0; r.ok && i < m; ++i) p.centers.push_back(r.f32s2());
  p.is_trained = r.u8() != 0;
  (void)r.u8();     // _has_residual
  (void)r.f32s();   // _residual
  (void)r.u64();    // _n_items
  (void)r.u64();    // _max_item
  read_nodes(r, p.nodes);  // _nodes (Box<Node> serialises as Node)
  (void)r.u64s2();  // _assigned_center (the codes; recomputed)
  p.mt = r.u32();
  Nodes tmp;
  read_nodes(r, tmp);  // _nodes_tmp (the dump's copy of _nodes)
  if (p.nodes.n == 0 && tmp.n) p.nodes = std::move(tmp);
  return r.ok;
}

int add_all(hora_index *h, const Nodes &nd) {
  if (nd.n == 0) return HORA_OK;
  return hora_add(h, nd.rows.data(), nd.ids.data(), nd.n);
}

// codebooks [C][M][K][dmax] from per-list [M][K][len] (dmax as the
// reference's ranges give it: dim / n_sub, plus one when it does not divide)
bool pack_books(const std::vector<std::vector<std::vector<float>>> &c, uint64_t n_sub, uint64_t K,
                uint64_t dmax, float *out) {
  if (c.empty()) return true;  // an untrained list stays zero
  if (c.size() != n_sub) return false;
  for (uint64_t m = 0; m < n_sub; ++m) {
    if (c[m].size() != K) return false;
    for (uint64_t j = 0; j < K; ++j) {
      if (c[m][j].size() > dmax) return false;
      std::memcpy(out + (m * K + j) * dmax, c[m][j].data(), 4 * c[m][j].size());
    }
  }
  return true;
}

int corrupt(const char *what) { return fail(HORA_EIO, std::string("reference index file: ") + what); }

}  // namespace

extern "C" {

int hora_load_reference(const char *path, int kind, hora_index **out) {
  if (!path || !out) return fail(HORA_EINVAL, "null argument");
  *out = nullptr;
  Reader r;
  {
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(HORA_EIO, std::string("unable to open file ") + path);
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
      std::fclose(f);
      return fail(HORA_EIO, std::string("unable to read file ") + path);
    }
    r.buf.resize((size_t)sz);
    const bool got = sz == 0 || std::fread(r.buf.data(), 1, (size_t)sz, f) == (size_t)sz;
    std::fclose(f);
    if (!got) return fail(HORA_EIO, std::string("unable to read file ") + path);
  }
  hora_index *h = nullptr;
  int rc = HORA_OK;
  if (kind == HORA_INDEX_BRUTE_FORCE) {
    // BruteForceIndex { nodes (skipped), tmp_nodes, mt, dimension } (bruteforce_idx.rs:15-21)
    Nodes nd;
    read_nodes(r, nd);
    const uint32_t mt = r.u32();
    const uint64_t dim = r.u64();
    if (!r.ok || dim == 0 || (nd.n && nd.dim != dim) || mt > HORA_METRIC_ANGULAR) return corrupt("BruteForceIndex");
    rc = hora_index_create(HORA_INDEX_BRUTE_FORCE, dim, nullptr, &h);
    if (rc == HORA_OK) rc = add_all(h, nd);
    if (rc == HORA_OK && mt != HORA_METRIC_UNKNOWN) rc = hora_build(h, (int)mt);
  } else if (kind == HORA_INDEX_PQ) {
    RefPQ p;
    if (!read_pq(r, p) || p.dimension == 0 || (p.nodes.n && p.nodes.dim != p.dimension) ||
        p.mt > HORA_METRIC_ANGULAR)
      return corrupt("PQIndex");
    hora_pq_params pp{p.n_sub, p.sub_bits, p.train_epoch};
    rc = hora_index_create(HORA_INDEX_PQ, p.dimension, &pp, &h);
    if (rc == HORA_OK) rc = add_all(h, p.nodes);
    if (rc == HORA_OK && p.is_trained && p.nodes.n) {
      if (p.mt == HORA_METRIC_COSINE_SIMILARITY || p.mt == HORA_METRIC_UNKNOWN || p.mt == HORA_METRIC_ANGULAR) {
        rc = fail(HORA_EMETRIC, "PQIndex: unsupported metric in the file");
      } else {
        h->metric = (int)p.mt;
        const uint64_t K = 1ull << p.sub_bits;
        const uint64_t sd = p.dimension / p.n_sub;
        const uint64_t dmax = sd + ((p.dimension % sd) ? 1 : 0);
        std::vector<float> books(p.n_sub * K * dmax, 0.0f), zero(p.dimension, 0.0f);
        if (!pack_books(p.centers, p.n_sub, K, dmax, books.data())) rc = corrupt("PQIndex codebooks");
        if (rc == HORA_OK) rc = hora_ivfpq_set_codebooks(h, zero.data(), books.data());
      }
    }
  } else if (kind == HORA_INDEX_IVFPQ) {
    // IVFPQIndex fields in declaration order (pq_idx.rs:266-289)
    const uint64_t dim = r.u64(), n_sub = r.u64();
    (void)r.u64();  // _sub_dimension
    const uint64_t sub_bits = r.u64();
    (void)r.u64();  // _sub_bytes
    (void)r.u64();  // _n_sub_center
    (void)r.u64();  // _code_bytes
    const uint64_t train_epoch = r.u64(), search_n_center = r.u64(), n_kmeans_center = r.u64();
    std::vector<std::vector<float>> centers = r.f32s2();
    std::vector<std::vector<uint64_t>> ivflist = r.u64s2();
    const uint64_t npq = r.len(8);
    std::vector<RefPQ> pqs(r.ok ? npq : 0);
    for (uint64_t c = 0; r.ok && c < npq; ++c) read_pq(r, pqs[c]);
    const bool trained = r.u8() != 0;
    (void)r.u64();  // _n_items
    (void)r.u64();  // _max_item
    Nodes nd;
    read_nodes(r, nd);  // _nodes
    (void)r.u64s2();    // _assigned_center
    const uint32_t mt = r.u32();
    Nodes tmp;
    read_nodes(r, tmp);  // _nodes_tmp
    if (nd.n == 0 && tmp.n) nd = std::move(tmp);
    if (!r.ok || dim == 0 || n_sub == 0 || (nd.n && nd.dim != dim) || mt > HORA_METRIC_ANGULAR)
      return corrupt("IVFPQIndex");
    hora_ivfpq_params ip{n_sub, sub_bits, n_kmeans_center, search_n_center, train_epoch};
    rc = hora_index_create(HORA_INDEX_IVFPQ, dim, &ip, &h);
    if (rc == HORA_OK) rc = add_all(h, nd);
    if (rc == HORA_OK && trained && nd.n) {
      const uint64_t C = n_kmeans_center, K = 1ull << sub_bits;
      const uint64_t sd = dim / n_sub, dmax = sd + ((dim % sd) ? 1 : 0);
      if (centers.size() != C || pqs.size() != C || ivflist.size() != C) {
        rc = corrupt("IVFPQIndex lists");
      } else {
        std::vector<float> cen(C * dim, 0.0f), books(C * n_sub * K * dmax, 0.0f);
        for (uint64_t c = 0; rc == HORA_OK && c < C; ++c) {
          if (centers[c].size() != dim) rc = corrupt("IVFPQIndex centres");
          else std::memcpy(cen.data() + c * dim, centers[c].data(), 4 * dim);
          if (rc == HORA_OK && !pack_books(pqs[c].centers, n_sub, K, dmax, books.data() + c * n_sub * K * dmax))
            rc = corrupt("IVFPQIndex codebooks");
        }
        h->metric = (int)mt;
        if (rc == HORA_OK) rc = hora_ivfpq_set_codebooks(h, cen.data(), books.data());
        if (rc == HORA_OK) {
          // the recomputed inverted lists must be the file's (same argmin)
          std::vector<int64_t> offs(C + 1), items(nd.n);
          rc = hora_ivfpq_export(h, nullptr, offs.data(), items.data(), nullptr, nullptr, nullptr);
          for (uint64_t c = 0; rc == HORA_OK && c < C; ++c) {
            const uint64_t L = (uint64_t)(offs[c + 1] - offs[c]);
            bool same = L == ivflist[c].size();
            for (uint64_t i = 0; same && i < L; ++i) same = (uint64_t)items[offs[c] + i] == ivflist[c][i];
            if (!same) rc = fail(HORA_EIO, "reference index file: the inverted lists disagree with the coarse assignment");
          }
        }
      }
    }
  } else {
    return fail(HORA_EINVAL, "unknown index kind");
  }
  if (rc != HORA_OK) {
    if (h) hora_index_free(h);
    return rc;
  }
  *out = h;
  return HORA_OK;
}

}  // extern "C"
