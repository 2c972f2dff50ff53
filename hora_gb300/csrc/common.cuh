// common.cuh — shared device helpers and host plumbing for libhora_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/hora_gb300.h"

namespace hora {

// ---- errors ---------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
extern std::atomic<uint64_t> g_launches;

#define HORA_CUDA_TRY(expr)                                                        \
  do {                                                                             \
    cudaError_t e__ = (expr);                                                      \
    if (e__ != cudaSuccess)                                                        \
      return ::hora::fail(e__ == cudaErrorMemoryAllocation ? HORA_EOOM : HORA_ECUDA, \
                          std::string(#expr) + ": " + cudaGetErrorString(e__));    \
  } while (0)

#define HORA_TRY(expr)           \
  do {                           \
    int rc__ = (expr);           \
    if (rc__ != HORA_OK) return rc__; \
  } while (0)

// Counts a launch and checks the launch error.
#define HORA_LAUNCHED()                                                           \
  do {                                                                            \
    ::hora::g_launches.fetch_add(1, std::memory_order_relaxed);                   \
    cudaError_t e__ = cudaGetLastError();                                         \
    if (e__ != cudaSuccess)                                                       \
      return ::hora::fail(HORA_ECUDA, std::string("launch: ") + cudaGetErrorString(e__)); \
  } while (0)

// ---- kernel timing ----------------------------------------------------------
// While profiling is on, a ProfScope records CUDA events around one launch on
// the launching stream; hora_profile_report() turns them into per-kernel time.
extern std::atomic<int> g_profile;
void prof_record(const char *name, cudaEvent_t a, cudaEvent_t b);
struct ProfScope {
  const char *name;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(const char *n, cudaStream_t st) : name(n), s(st) {
    if (g_profile.load(std::memory_order_relaxed)) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEventRecord(b, s);
      prof_record(name, a, b);
    }
  }
};

// ---- metric ids ------------------------------------------------------------
enum MetricId : int {
  M_UNKNOWN = HORA_METRIC_UNKNOWN,
  M_L1 = HORA_METRIC_MANHATTAN,
  M_IP = HORA_METRIC_DOT_PRODUCT,
  M_L2 = HORA_METRIC_EUCLIDEAN,
  M_COS = HORA_METRIC_COSINE_SIMILARITY,
};

// ---- sort keys ---------------------------------------------------------------
// A candidate is one 64-bit key: the order-preserving image of its f32
// distance in the high word and its row number in the low word, so that an
// unsigned compare orders by (distance, row) — ties go to the lower row.
constexpr uint64_t kEmptyKey = ~0ull;

__host__ __device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  memcpy(&u, &f, 4);
#endif
  if (u == 0x80000000u) u = 0;                             // -0 == +0
  if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu)) u = 0x7fc00000u;  // one NaN, after +inf
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ __forceinline__ float ord2f(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
#ifdef __CUDA_ARCH__
  f = __uint_as_float(u);
#else
  memcpy(&f, &u, 4);
#endif
  return f;
}

__host__ __device__ __forceinline__ uint64_t make_key(float d, uint32_t row) {
  return ((uint64_t)f2ord(d) << 32) | row;
}
__host__ __device__ __forceinline__ float key_dist(uint64_t k) { return ord2f((uint32_t)(k >> 32)); }
__host__ __device__ __forceinline__ uint32_t key_row(uint64_t k) { return (uint32_t)k; }

// ---- the splitmix64 stream (shared with the oracle) ----------------------------
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t instance_seed(uint64_t seed, uint64_t inst) {
  return mix64(seed ^ mix64(inst * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull));
}
constexpr uint64_t kRngStep = 0x9E3779B97F4A7C15ull;

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// ---- device memory -------------------------------------------------------------
// Grow-only device buffer owned by an index or a search context.
// Page-locked host memory: the target of asynchronous device-to-host copies.
struct HostBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  HostBuf() = default;
  HostBuf(const HostBuf &) = delete;
  HostBuf &operator=(const HostBuf &) = delete;
  ~HostBuf() {
    if (ptr) cudaFreeHost(ptr);
  }
  int reserve(size_t want) {
    if (want <= bytes) return HORA_OK;
    void *p = nullptr;
    if (cudaHostAlloc(&p, want, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return fail(HORA_EOOM, "cudaHostAlloc failed");
    }
    if (ptr) cudaFreeHost(ptr);
    ptr = p;
    bytes = want;
    return HORA_OK;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

// An event created on first use and destroyed with its owner.
struct EventBox {
  cudaEvent_t ev = nullptr;
  EventBox() = default;
  EventBox(const EventBox &) = delete;
  EventBox &operator=(const EventBox &) = delete;
  ~EventBox() {
    if (ev) cudaEventDestroy(ev);
  }
  int ensure(bool timing = false) {
    if (ev) return HORA_OK;
    if (cudaEventCreateWithFlags(&ev, timing ? cudaEventDefault : cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      ev = nullptr;
      return fail(HORA_ECUDA, "cudaEventCreate failed");
    }
    return HORA_OK;
  }
};

struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  // Ensures capacity; contents are not preserved unless keep is set.
  int reserve(size_t want, cudaStream_t s = 0, bool keep = false) {
    if (want <= bytes) return HORA_OK;
    size_t cap = want < 256 ? 256 : want;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, cap);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(HORA_EOOM, std::string("cudaMalloc(") + std::to_string(cap) + "): " + cudaGetErrorString(e));
    }
    if (keep && ptr && bytes) {
      e = cudaMemcpyAsync(p, ptr, bytes, cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        cudaFree(p);
        return fail(HORA_ECUDA, std::string("grow copy: ") + cudaGetErrorString(e));
      }
    }
    release();
    ptr = p;
    bytes = cap;
    return HORA_OK;
  }
  template <class T>
  T *as() const { return reinterpret_cast<T *>(ptr); }
};

// Where a caller's buffer lives.  PTR_HOST: host memory (pageable or
// page-locked), copied by the library.  PTR_DEVICE: memory the current
// device's kernels may read and write in place (its own allocations or
// managed memory).  PTR_FOREIGN: device memory of another device, which
// the library's kernels must not touch (without peer access that faults).
enum PtrKind : int { PTR_FOREIGN = -1, PTR_HOST = 0, PTR_DEVICE = 1 };
int pointer_kind(const void *p);
// pointer_kind(p) == PTR_DEVICE
bool is_device_ptr(const void *p);
// HORA_EINVAL when p is memory of another device (null passes).
int check_not_foreign(const void *p, const char *what);

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The attribute belongs to each device's context, so it is
// tracked per (kernel, device): a process-wide flag would leave every device
// after the first without it.
int ensure_smem_attr(const void *kernel, int bytes);
#define HORA_SMEM_ATTR(kernel, bytes) \
  HORA_TRY(::hora::ensure_smem_attr(reinterpret_cast<const void *>(kernel), (int)(bytes)))

}  // namespace hora
