// noalloc.cu — exact brute-force k-NN that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host engine that owns every byte of
// device memory through its own pool and hard budget, or a latency-critical
// request path where cudaMalloc / cudaFree would synchronise the device and
// stall other streams.  hora_bf_search_noalloc serves them: the caller
// passes the base, the queries and the outputs in device memory, and every
// piece of scratch the search needs (per-query k-best lists, candidate
// buffers, counters) lives in one file-scope __device__ array of fixed size,
// present on every GPU that loads the library until the process exits.
//
// Limits: at most kNaMaxQueries queries and k <= kNaMaxK per call; dim a
// multiple of 4 with 16-byte aligned rows; Euclidean, Manhattan or
// DotProduct (cosine would need per-row norms of the whole base).  Every
// buffer must be memory of the current device (or managed memory).  A NaN or
// Inf element in the queries or the base is HORA_ENAN, as hora_search and
// hora_add report it (the reference panics, src/core/node.rs:158-166); the
// flag is read before any result is written.
// All calls share the array and it keeps the previous call's contents, so
// this code clears what must start at zero on every call, and two calls that
// overlap on the GPU (different streams or threads) race on it.  A call is
// synchronous: it waits on its stream and returns once the results are in
// the caller's buffers.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (the host-side name is only a stand-in for it) and
// caches it per device; make that first call before any stream capture.
#include <mutex>

#include "internal.h"

namespace hora {
namespace {

constexpr int kNaMaxQueries = 256;
constexpr int kNaMaxK = 64;
constexpr int kNaCap = 1024;  // candidates per query per chunk
constexpr int kNaMaxDevices = 64;

struct NaScratch {
  uint64_t best[kNaMaxQueries * kNaMaxK];
  uint64_t cand[kNaMaxQueries * kNaCap];
  uint32_t count[kNaMaxQueries];
  int qlist[kNaMaxQueries];
  uint8_t flags[kNaMaxQueries];
  uint32_t ovf_counter[4];  // [0] overflowed queries, [1] non-finite input element
  uint32_t nlist[4];
};

}  // namespace

// 2.1 MiB per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NaScratch)];

static std::mutex g_na_mu;
static NaScratch *g_na_addr[kNaMaxDevices];

static int noalloc_scratch(NaScratch **out) {
  int dev = 0;
  HORA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) return fail(HORA_ECAP, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_na_mu);
  if (!g_na_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(HORA_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_na_addr[dev] = reinterpret_cast<NaScratch *>(p);
  }
  *out = g_na_addr[dev];
  return HORA_OK;
}

// Collects the queries whose candidates overflowed into qlist (any order)
// and clears their flags.
__global__ void noalloc_collect_kernel(uint8_t *flags, int nq, int *qlist, uint32_t *nlist) {
  for (int q = threadIdx.x; q < nq; q += blockDim.x)
    if (flags[q]) {
      qlist[atomicAdd(nlist, 1u)] = q;
      flags[q] = 0;
    }
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace hora

using namespace hora;

extern "C" int hora_bf_search_noalloc(const float *base, uint64_t n, uint64_t dim,
                                      const float *queries, uint64_t nq, uint64_t k, int metric,
                                      uint64_t *ids_out, float *dist_out, void *stream) {
  if (!base || !queries || !ids_out || !dist_out) return fail(HORA_EINVAL, "null buffer");
  if (metric != M_L2 && metric != M_L1 && metric != M_IP)
    return fail(HORA_EMETRIC, "noalloc search supports Euclidean, Manhattan and DotProduct");
  if (nq == 0) return HORA_OK;
  if (nq > (uint64_t)kNaMaxQueries)
    return fail(HORA_ECAP, "noalloc search: at most 256 queries per call");
  if (k == 0) return fail(HORA_EINVAL, "k must be positive");
  if (k > (uint64_t)kNaMaxK) return fail(HORA_ECAP, "noalloc search: k must be <= 64");
  if (dim == 0 || dim % 4) return fail(HORA_EINVAL, "noalloc search: dim must be a multiple of 4");
  if (n == 0 || n >= (uint64_t)UINT32_MAX) return fail(HORA_ECAP, "noalloc search: n must be in [1, 2^32-1)");
  if (!aligned16(base) || !aligned16(queries))
    return fail(HORA_EINVAL, "noalloc search: base and queries must be 16-byte aligned");
  if (!is_device_ptr(base) || !is_device_ptr(queries) || !is_device_ptr(ids_out) ||
      !is_device_ptr(dist_out))
    return fail(HORA_EINVAL, "noalloc search: all buffers must be memory of the current device");
  NaScratch *sc = nullptr;
  HORA_TRY(noalloc_scratch(&sc));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int K = (int)k, Q = (int)nq;
  // the array keeps the previous call's contents: reset what starts empty
  HORA_CUDA_TRY(cudaMemsetAsync(sc->best, 0xff, sizeof(uint64_t) * Q * K, s));
  HORA_CUDA_TRY(cudaMemsetAsync(sc->count, 0, sizeof(uint32_t) * Q, s));
  HORA_CUDA_TRY(cudaMemsetAsync(sc->flags, 0, Q, s));
  HORA_CUDA_TRY(cudaMemsetAsync(sc->ovf_counter, 0, sizeof(sc->ovf_counter), s));
  const int64_t N = (int64_t)n;
  HORA_TRY(launch_check_finite(queries, Q, (int64_t)dim, (int64_t)dim, &sc->ovf_counter[1], s));
  HORA_TRY(launch_check_finite(base, N, (int64_t)dim, (int64_t)dim, &sc->ovf_counter[1], s));

  TileParams p;
  p.Q = queries;
  p.ldq = (int64_t)dim;
  p.nq = Q;
  p.X = base;
  p.ldx = (int64_t)dim;
  p.ld = (int64_t)dim;
  p.best = sc->best;
  p.k = K;
  p.cand = sc->cand;
  p.cap = kNaCap;
  p.count = sc->count;
  const int64_t c0 = N < kNaCap ? N : kNaCap;
  p.r_begin = 0;
  p.r_end = c0;
  HORA_TRY(launch_dist_tile(metric, TILE_DENSE, p, s));
  HORA_TRY(launch_merge_topk(sc->best, K, sc->cand, sc->count, kNaCap, (int)c0, nullptr, Q,
                             sc->flags, sc->ovf_counter, s));
  int64_t done = c0;
  const int64_t max_chunk = (int64_t)65535 * 128;
  while (done < N) {
    double grow = (double)kNaCap / (4.0 * K);
    int64_t c = (int64_t)((double)done * (grow > 1.0 ? grow : 1.0));
    if (c < 128 * 64) c = 128 * 64;
    c = round_up(c, 128);
    if (c > N - done) c = N - done;
    if (c > max_chunk) c = max_chunk;
    p.r_begin = done;
    p.r_end = done + c;
    HORA_TRY(launch_dist_tile(metric, TILE_FILTER, p, s));
    HORA_TRY(launch_merge_topk(sc->best, K, sc->cand, sc->count, kNaCap, 0, nullptr, Q, sc->flags,
                               sc->ovf_counter, s));
    done += c;
  }
  // the input check, then a rescan of the queries whose candidates
  // overflowed, with their tightened bound
  uint32_t st[2] = {0, 0};
  HORA_CUDA_TRY(cudaMemcpyAsync(st, sc->ovf_counter, sizeof(st), cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  if (st[1]) return fail(HORA_ENAN, "invalid float element");
  uint32_t ovc = st[0];
  for (int round = 0; ovc > 0; ++round) {
    if (round >= 64) return fail(HORA_ECUDA, "noalloc search: overflow rescan did not converge");
    HORA_CUDA_TRY(cudaMemsetAsync(sc->nlist, 0, sizeof(sc->nlist), s));
    noalloc_collect_kernel<<<1, 256, 0, s>>>(sc->flags, Q, sc->qlist, sc->nlist);
    HORA_LAUNCHED();
    uint32_t nl = 0;
    HORA_CUDA_TRY(cudaMemcpyAsync(&nl, sc->nlist, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaMemsetAsync(sc->ovf_counter, 0, sizeof(sc->ovf_counter), s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    TileParams r = p;
    r.nq = nl;
    r.qmap = sc->qlist;
    for (int64_t lo = 0; lo < N; lo += max_chunk) {
      r.r_begin = lo;
      r.r_end = lo + max_chunk < N ? lo + max_chunk : N;
      HORA_TRY(launch_dist_tile(metric, TILE_FILTER, r, s));
      HORA_TRY(launch_merge_topk(sc->best, K, sc->cand, sc->count, kNaCap, 0, sc->qlist, nl,
                                 sc->flags, sc->ovf_counter, s));
    }
    HORA_CUDA_TRY(cudaMemcpyAsync(&ovc, sc->ovf_counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  HORA_TRY(launch_keys_to_results(sc->best, (int64_t)Q * K, nullptr, ids_out, dist_out, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  return HORA_OK;
}
