// runtime.cu -- error reporting, scratch memory, problem validation.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace epet {

// Device memory of the library comes from one stream-ordered pool per
// device that keeps freed memory reserved (release threshold: unlimited), so
// a reconstruction set up again with the same sizes maps no new memory;
// epet_trim_memory hands the reserve back.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[64] = {};

static cudaMemPool_t lib_pool(cudaError_t* err) {
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    *err = cudaMemPoolCreate(&g_pool[dev], &props);
    if (*err != cudaSuccess) {
      g_pool[dev] = nullptr;
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
  }
  return g_pool[dev];
}

static std::atomic<long long> g_allocs{0};

// Host-side fault injection for tests of the error paths: after this many
// more allocations (-1: never) every device allocation of the library fails
// with cudaErrorMemoryAllocation.  Nothing reaches the device.
static std::atomic<long long> g_fail_after{-1};

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t st) {
  long long left = g_fail_after.load(std::memory_order_relaxed);
  while (left >= 0) {
    if (left == 0) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
    if (g_fail_after.compare_exchange_weak(left, left - 1, std::memory_order_relaxed)) break;
  }
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaSuccess;
  cudaMemPool_t pool = lib_pool(&e);
  if (!pool) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

cudaError_t dev_free(void* p, cudaStream_t st) { return cudaFreeAsync(p, st); }

epet_status trim_memory(size_t keep_bytes) {
  std::lock_guard<std::mutex> lock(g_pool_mu);
  for (int d = 0; d < 64; d++) {
    if (!g_pool[d]) continue;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(d);
    cudaDeviceSynchronize();
    cudaError_t e = cudaMemPoolTrimTo(g_pool[d], keep_bytes);
    cudaSetDevice(cur);
    if (e != cudaSuccess) return cuda_status(e, "cudaMemPoolTrimTo");
  }
  return EPET_OK;
}

static thread_local char g_err[512] = "";

epet_status set_error(epet_status st, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return st;
}

epet_status cuda_status(cudaError_t e, const char* what) {
  return set_error(EPET_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

epet_status Scratch::init(void* ws, size_t ws_bytes, size_t need,
                          cudaStream_t s) {
  stream = s;
  size = need;
  used = 0;
  if (need == 0) return EPET_OK;
  if (ws) {
    if (ws_bytes < need)
      return set_error(EPET_ERR_CAPACITY,
                       "workspace too small: %zu bytes given, %zu needed",
                       ws_bytes, need);
    if (reinterpret_cast<uintptr_t>(ws) & 255)
      return set_error(EPET_ERR_INVALID, "workspace must be 256-byte aligned");
    base = static_cast<char*>(ws);
    owned = false;
    return EPET_OK;
  }
  cudaError_t e = dev_alloc(reinterpret_cast<void**>(&base), need, s);
  if (e != cudaSuccess) {
    base = nullptr;
    return cuda_status(e, "workspace allocation");
  }
  owned = true;
  return EPET_OK;
}

Scratch::~Scratch() {
  if (owned && base) dev_free(base, stream);
}

static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches() { return g_launches.load(); }

int num_sms() {  // of the current device, cached per device (any thread)
  static std::atomic<int> cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int>* slot = dev >= 0 && dev < 64 ? &cache[dev] : nullptr;
  int n = slot ? slot->load(std::memory_order_relaxed) : 0;
  if (n == 0) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
    if (slot) slot->store(n, std::memory_order_relaxed);
  }
  return n;
}

}  // namespace epet

extern "C" {

const char* epet_last_error(void) { return epet::g_err; }

const char* epet_version(void) { return "epet_gb300 1.0 (sm_103a)"; }

long long epet_launch_count(void) { return epet::launches(); }

epet_status epet_debug_fail_allocations(long long after) {
  epet::g_fail_after.store(after < 0 ? -1 : after, std::memory_order_relaxed);
  return EPET_OK;
}

long long epet_device_allocations(void) { return epet::g_allocs.load(); }

epet_status epet_problem_validate(const epet_problem* p) {
  using epet::set_error;
  if (!p) return set_error(EPET_ERR_INVALID, "problem is NULL");
  const epet_setup& s = p->setup;
  const epet_grid& g = p->grid;
  if (p->nrays < 1) return set_error(EPET_ERR_INVALID, "nrays must be >= 1");
  if (p->ray_mode != EPET_RAYS_RANDOM && p->ray_mode != EPET_RAYS_REGULAR)
    return set_error(EPET_ERR_INVALID, "ray_mode must be EPET_RAYS_RANDOM or EPET_RAYS_REGULAR");
  if (s.na < 1 || s.n0z < 1 || s.n0y < 1 || s.n1z < 1 || s.n1y < 1)
    return set_error(EPET_ERR_INVALID, "detector counts must be >= 1");
  double nch = (double)s.na * s.n0z * s.n0y * s.n1z * s.n1y;
  if (nch > 2147483647.0)
    return set_error(EPET_ERR_UNSUPPORTED, "channel count exceeds int32");
  for (int d = 0; d < 3; d++) {
    if (g.n[d] < 1) return set_error(EPET_ERR_INVALID, "grid counts must be >= 1");
    if (!(g.d[d] > 0.f)) return set_error(EPET_ERR_INVALID, "grid pitch must be > 0");
  }
  double V = (double)g.n[0] * g.n[1] * g.n[2];
  if (V > 2147483647.0)
    return set_error(EPET_ERR_UNSUPPORTED, "voxel count exceeds int32");
  if (!(s.segx > 0.f && s.segy > 0.f && s.segz > 0.f))
    return set_error(EPET_ERR_INVALID, "crystal edges must be > 0");
  return EPET_OK;
}

}  // extern "C"
