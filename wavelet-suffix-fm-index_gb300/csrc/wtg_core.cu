// wtg_core.cu -- error reporting, stream-ordered device buffers, launch
// accounting and the generic single-pass exclusive scan used by the build.
#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "wtg_internal.cuh"

namespace wtg {

WTG_WAIT_LIMIT_SETTER(core)

static thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return WTG_ERR_OOM;
  return WTG_ERR_CUDA;
}

// Keep freed stream-ordered allocations cached in the device pool so that
// repeated builds of the same shape do not return memory to the driver.
static int ensure_pool_setup() {
  static std::once_flag once;
  static cudaError_t status = cudaSuccess;
  std::call_once(once, [] {
    int dev = 0;
    status = cudaGetDevice(&dev);
    if (status != cudaSuccess) return;
    cudaMemPool_t pool;
    status = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (status != cudaSuccess) return;
    uint64_t thr = ~0ull;
    status = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  });
  if (status != cudaSuccess) return cuda_fail(status, "device memory pool setup");
  return WTG_OK;
}

// ------------------------------------------------------- test hooks
// Failure injection on the host side only: an armed countdown makes one
// device allocation report WTG_ERR_OOM, and an armed stall makes the next
// rank/select pass's look-back waits run out (see wtg_internal.cuh).
static std::atomic<int64_t> g_alloc_fail_countdown{0};
static std::atomic<int> g_lookback_stall{0};

void test_arm_alloc_failure(int64_t nth) { g_alloc_fail_countdown.store(nth > 0 ? nth : 0); }
void test_arm_lookback_stall(int on) { g_lookback_stall.store(on ? 1 : 0); }

bool test_take_alloc_failure() {
  int64_t c = g_alloc_fail_countdown.load();
  while (c > 0)
    if (g_alloc_fail_countdown.compare_exchange_weak(c, c - 1)) return c == 1;
  return false;
}

bool test_take_lookback_stall() {
  int armed = 1;
  return g_lookback_stall.compare_exchange_strong(armed, 0);
}

int DevBuf::ensure(size_t need, cudaStream_t s) {
  if (need <= bytes && p) return WTG_OK;
  int rc = ensure_pool_setup();
  if (rc) return rc;
  // an injected failure leaves the buffer as it was, like a failed cudaMallocAsync
  if (test_take_alloc_failure()) return fail(WTG_ERR_OOM, "device allocation failed (injected by wtg_test_fail_alloc)");
  if (p) {
    cudaFreeAsync(p, s);
    p = nullptr;
    bytes = 0;
  }
  size_t alloc = need ? need : 16;
  cudaError_t e = cudaMallocAsync(&p, alloc, s);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMallocAsync");
  }
  bytes = alloc;
  return WTG_OK;
}

void DevBuf::release(cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
  p = nullptr;
  bytes = 0;
}

// ------------------------------------------------------------- profiling

struct ProfRec {
  int cls;
  cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof;
static std::vector<cudaEvent_t> g_prof_free;
static std::atomic<bool> g_prof_enabled{false};
static thread_local cudaEvent_t t_prof_open = nullptr;

static cudaEvent_t prof_event() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_free.empty()) {
    cudaEvent_t e = g_prof_free.back();
    g_prof_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

bool prof_on() { return g_prof_enabled.load(std::memory_order_relaxed); }

void prof_begin(int, cudaStream_t s) {
  if (!prof_on()) return;
  t_prof_open = prof_event();
  cudaEventRecord(t_prof_open, s);
}

void prof_end(int cls, cudaStream_t s) {
  if (!prof_on() || !t_prof_open) return;
  cudaEvent_t b = prof_event();
  cudaEventRecord(b, s);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.push_back({cls, t_prof_open, b});
  t_prof_open = nullptr;
}

// ------------------------------------------------------------------ scan

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS)
    scan_exclusive_kernel(const T* __restrict__ in, T* __restrict__ out, uint64_t n, uint64_t* status,
                          uint32_t* counter, uint32_t* err) {
  __shared__ uint32_t s_tile;
  __shared__ uint64_t s_wsum[SCAN_THREADS / 32];
  __shared__ uint64_t s_prefix;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t base = (uint64_t)tile * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_IPT;
  uint64_t v[SCAN_IPT];
  uint64_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint64_t idx = base + k;
    v[k] = idx < n ? (uint64_t)in[idx] : 0;
    sum += v[k];
  }
  uint64_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) s_wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < SCAN_THREADS / 32 ? s_wsum[lane] : 0;
    uint64_t winc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t t = __shfl_up_sync(0xffffffffu, winc, o);
      if (lane >= (uint32_t)o) winc += t;
    }
    if (lane < SCAN_THREADS / 32) s_wsum[lane] = winc - w;
    uint64_t total = __shfl_sync(0xffffffffu, winc, SCAN_THREADS / 32 - 1);
    uint64_t prefix = 0;
    if (tile == 0) {
      if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, total);
    } else {
      if (lane == 0) lb_publish(status, tile, LB_FLAG_AGG, total);
      prefix = lb_lookback_warp(status, tile, err);
      if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, prefix + total);
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  uint64_t run = s_prefix + s_wsum[warp] + incl - sum;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint64_t idx = base + k;
    if (idx < n) out[idx] = (T)run;
    run += v[k];
  }
}

template <typename T>
static int scan_exclusive(const T* in, T* out, uint64_t n, DevBuf& scratch, uint32_t* d_err, cudaStream_t s) {
  if (n == 0) return WTG_OK;
  uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles > 0x7fffffffull) return fail(WTG_ERR_INVALID, "scan too large");
  size_t bytes = (tiles + 1) * sizeof(uint64_t);
  int rc = scratch.ensure(bytes, s);
  if (rc) return rc;
  WTG_CK(cudaMemsetAsync(scratch.p, 0, bytes, s));
  uint64_t* status = scratch.as<uint64_t>() + 1;
  uint32_t* counter = scratch.as<uint32_t>();
  prof_begin(PROF_TABLES, s);
  scan_exclusive_kernel<T><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, status, counter, d_err);
  prof_end(PROF_TABLES, s);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n, DevBuf& scratch, uint32_t* d_err,
                       cudaStream_t s) {
  return scan_exclusive<uint32_t>(in, out, n, scratch, d_err, s);
}
int scan_exclusive_u64(const uint64_t* in, uint64_t* out, uint64_t n, DevBuf& scratch, uint32_t* d_err,
                       cudaStream_t s) {
  return scan_exclusive<uint64_t>(in, out, n, scratch, d_err, s);
}

}  // namespace wtg

extern "C" {
int wtg_profile_enable(int on) {
  wtg::g_prof_enabled.store(on != 0);
  return WTG_OK;
}

int wtg_profile_read(uint64_t launches[WTG_PROF_CLASSES], double ms[WTG_PROF_CLASSES]) {
  using namespace wtg;
  std::vector<ProfRec> recs;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    recs.swap(g_prof);
  }
  for (int c = 0; c < WTG_PROF_CLASSES; ++c) {
    if (launches) launches[c] = 0;
    if (ms) ms[c] = 0.0;
  }
  int rc = WTG_OK;
  for (auto& r : recs) {
    cudaError_t e = cudaEventSynchronize(r.b);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.a, r.b);
    if (e != cudaSuccess && rc == WTG_OK) rc = cuda_fail(e, "profile events");
    if (r.cls >= 0 && r.cls < WTG_PROF_CLASSES) {
      if (launches) launches[r.cls] += 1;
      if (ms) ms[r.cls] += t;
    }
  }
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& r : recs) {
    g_prof_free.push_back(r.a);
    g_prof_free.push_back(r.b);
  }
  return rc;
}

const char* wtg_last_error(void) { return wtg::g_last_error.c_str(); }
int wtg_version(void) { return 100; }
uint64_t wtg_launch_count(void) { return wtg::g_launches.load(); }
}
