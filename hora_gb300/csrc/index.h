// index.h — the handle behind hora_index* (shared by the translation units).
#pragma once

#include <atomic>
#include <memory>
#include <mutex>

#include "internal.h"

namespace hora {

struct IvfState;   // ivfpq.cu
struct LowpState;  // bf_lowp.cu
struct CoarseTc;   // bf_lowp.cu
struct NprobeModel;  // nprobe_mlp.cu

void ivf_state_free(IvfState *);
void lowp_state_free(LowpState *);
void coarse_tc_free(CoarseTc *);
void nprobe_model_free(NprobeModel *);
struct IvfDeleter { void operator()(IvfState *p) const { ivf_state_free(p); } };
struct LowpDeleter { void operator()(LowpState *p) const { lowp_state_free(p); } };
struct CoarseTcDeleter { void operator()(CoarseTc *p) const { coarse_tc_free(p); } };
struct NprobeDeleter { void operator()(NprobeModel *p) const { nprobe_model_free(p); } };

}  // namespace hora

struct hora_index {
  int kind = HORA_INDEX_BRUTE_FORCE;
  uint64_t dim = 0, ld = 0;  // ld: row pitch in floats (dim rounded up to 4, zero padded)
  hora_ivfpq_params ivf{};
  int metric = HORA_METRIC_UNKNOWN;
  bool built = false;
  int64_t n = 0, cap_rows = 0;
  hora::DevBuf base;  // cap_rows x ld f32, insertion order
  hora::DevBuf ids;   // cap_rows u64 user ids
  hora::DevBuf xnorm; // n f32 sqrt norms (cosine)
  hora::DevBuf xsq64; // n f64 squared norms (GEMM forms)
  bool norms_valid = false;

  // GPU-only options
  int precision = HORA_PREC_FP32;
  int rerank = 0;
  int cand_cap = 4096;
  int accum_f64 = 1;
  uint64_t seed = 0x686f7261ull;
  uint64_t train_size = 0;
  int learned_nprobe = 0;
  double nprobe_margin = 0.0;
  int nprobe_max = 0;
  int ivf_rerank = 0;
  int nprobe_phase1 = 4;
  int bf_probe = 1;
  int exact_tc = 1;

  cudaStream_t stream = nullptr;
  std::mutex mu;
  hora::SearchWorkspace ws;
  std::unique_ptr<hora::IvfState, hora::IvfDeleter> ivfs;
  std::unique_ptr<hora::LowpState, hora::LowpDeleter> lowp;
  // the IVF centres' BF16 image for the certified coarse probe (bf_lowp.cu)
  std::unique_ptr<hora::CoarseTc, hora::CoarseTcDeleter> coarse_tc;
  std::unique_ptr<hora::NprobeModel, hora::NprobeDeleter> nprobe;
  // last search diagnostics (written by whichever search finished last)
  std::atomic<int> last_retries{0};
  // BF16 starting-threshold probe: 0 not used, 1 answered, 2 fell back to the chunked schedule
  std::atomic<int> last_probe{0};
  // low-precision search: queries whose candidate list overflowed its
  // capacity (before the rescans), queries the probed pass left short
  std::atomic<int64_t> last_overflow_queries{0}, last_short_lists{0};
  // certified exact search: queries the last search handed to the CUDA-core scan
  std::atomic<int64_t> last_fallback{0};
  std::atomic<double> last_ms{0.0};
};

namespace hora {

BaseView base_view(hora_index *h);
int search_core(hora_index *h, SearchWorkspace &ws, cudaStream_t s, const float *queries,
                uint64_t nq, uint64_t k, uint64_t nprobe, uint64_t *ids_out, float *dist_out,
                float *vecs_out);
// Builds the lazily derived state a search may need (norms, low-precision
// copy) so that concurrent searches only read the index.
int prepare_for_concurrent_search(hora_index *h);
int ensure_norms(hora_index *h, cudaStream_t s);
// Copies nq x dim queries (host or device) into ws.q with pitch h->ld, checks
// finiteness and computes f32 norms when the metric needs them.  With
// defer_check, the queries (host or device) are checked on the device and the
// flag is copied to ws.h_status behind ws.ev_status without waiting; the
// caller reads it before it writes any result.
int stage_queries(hora_index *h, const float *queries, int64_t nq, SearchWorkspace &ws,
                  cudaStream_t s, bool defer_check = false);

// Brute force with the handle's precision option; writes nq x k keys.
int bf_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                   cudaStream_t s);

// Low-precision scoring + FP32 rerank (bf_lowp.cu).
int lowp_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                     cudaStream_t s);
int lowp_prepare(hora_index *h, cudaStream_t s);
// Candidates a low-precision search keeps for its exact rerank (0 when the
// exact path answers: Manhattan, or dimensions beyond the resident tile).
int lowp_rerank_width(const hora_index *h, int k);
// The starting threshold a low-precision search of an R-best list takes: 0
// none (the chunked schedule), 1 the cluster probe, 2 the sampled threshold.
int lowp_probe_kind(const hora_index *h, int R);
// Exact FP32 Euclidean search with the BF16 tensor-core scan as a certified
// filter (bf_lowp.cu): whether it answers a k-NN search on this index, its
// lazily built state, the search itself.
bool exact_tc_eligible(const hora_index *h, int k);
// The IVF coarse probe on the tensor cores (bf_lowp.cu): each query's pmax
// nearest centres (ascending exact keys, the FP32 probe's result), from a
// BF16 pass over the centres and an exact rescoring of the centres within
// the certified error bound of the pmax-th; dist is nq x C scratch.
bool coarse_tc_eligible(const hora_index *h);
int coarse_tc_probe(hora_index *h, const float *centers, const float *cnorm, int64_t C, int64_t nq, int pmax,
                    SearchWorkspace &ws, float *dist, uint64_t *probes, cudaStream_t s);
int exact_tc_prepare(hora_index *h, cudaStream_t s);
int exact_tc_search_keys(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                         cudaStream_t s);

// IVF-PQ (ivfpq.cu)
int ivf_build(hora_index *h);
int ivf_search_keys(hora_index *h, int64_t nq, int k, int64_t nprobe, const uint32_t *d_nprobe,
                    SearchWorkspace &ws, uint64_t *d_best, cudaStream_t s);
int ivf_pmax(const hora_index *h, int64_t nprobe);
int ivf_probe(hora_index *h, int64_t nq, int pmax, SearchWorkspace &ws, cudaStream_t s);
const uint64_t *ivf_probe_keys(const SearchWorkspace &ws);
int ivf_adc_merge(hora_index *h, int64_t nq, int pmax, int jbegin, const uint32_t *d_nprobe,
                  int R, uint64_t *M, SearchWorkspace &ws, cudaStream_t s);
int ivf_finalize(hora_index *h, int64_t nq, int k, int R, const uint64_t *M, SearchWorkspace &ws,
                 uint64_t *d_best, cudaStream_t s);
int ivf_rerank_width(const hora_index *h, int k);
uint64_t *ivf_merge_buffer(SearchWorkspace &ws, int64_t nq, int R, uint64_t *d_best, int k);
// learned nprobe (nprobe_mlp.cu)
int ivf_search_learned(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                       cudaStream_t s);
// JSON of the trained nprobe model (phase-1 probes, calibrated margin and
// its held-out recall / mean nprobe), "null" without a model
std::string nprobe_model_info(const hora_index *h);
int ivf_layout(const hora_index *h, uint64_t *n_list, uint64_t *n_sub, uint64_t *sub_bits,
               uint64_t *dmax);
int ivf_export(const hora_index *h, float *centers, int64_t *offsets, int64_t *items,
               float *codebooks, uint8_t *codes, uint8_t *trained);
int ivf_set_codebooks(hora_index *h, const float *centers, const float *codebooks);
int ivf_dump(const hora_index *h, FILE *f);
int ivf_load(hora_index *h, FILE *f);
size_t ivf_device_bytes(const hora_index *h);
int ivf_info(const hora_index *h, std::string &out);

}  // namespace hora
