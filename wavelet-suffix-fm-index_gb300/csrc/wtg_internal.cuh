// wtg_internal.cuh -- device primitives and internal host interfaces shared by
// the wtg CUDA sources (GB300 / sm_103a).
//
// Data layouts kept bit-exact with the reference (jlabeit/wavelet-suffix-fm-index):
//   * level bitvector: level l occupies bits [l*n, (l+1)*n) of one array of
//     64-bit words, LSB first (wavelet/levelWT/WT.C:54,61,93);
//   * rank_support_v<1> table: interleaved (absolute count, seven 9-bit
//     cumulative block counts) per 512-bit superblock
//     (rank/rank_support_v_par.hpp:78-113);
//   * select_support_mcl<t_b>: m_superblock int_vector<0> of width logn, and
//     per superblock a 64-entry mini block or a 4096-entry long block
//     (select/select_support_mcl_par.hpp:483-561), stored flat (see
//     include/wtg.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/wtg.h"

namespace wtg {

// number of kernel launches issued (reported through wtg_launch_count)
extern std::atomic<uint64_t> g_launches;
inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// kernel-class profiling (wtg_profile_enable / wtg_profile_read)
enum ProfClass { PROF_LEVEL = 0, PROF_LEVEL_LAST, PROF_HIST, PROF_TABLES, PROF_BVPASS, PROF_SELECT, PROF_N };
bool prof_on();
void prof_begin(int cls, cudaStream_t s);  // call right before a launch
void prof_end(int cls, cudaStream_t s);    // call right after it

// ------------------------------------------------------------------ errors

// Device-side error codes written to the per-handle error word.
enum : uint32_t {
  DERR_NONE = 0,
  DERR_LOOKBACK_TIMEOUT = 1,  // a decoupled look-back wait gave up
  DERR_BAD_SYMBOL = 2,
  DERR_SELECT_OVERFLOW = 3,  // more args in a superblock than fit its block
  DERR_BAD_INDEX = 4,        // a computed destination fell outside its buffer
};

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define WTG_CK(call)                                   \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return ::wtg::cuda_fail(_e, #call); \
  } while (0)

// ------------------------------------------------------ device primitives

constexpr uint64_t NONE64 = ~0ull;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// position of the r-th (0-based) set bit of x, r < popc(x); branch-free
// halving search over popcounts
__device__ __forceinline__ uint32_t sel64_0(uint64_t x, uint32_t r) {
  const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
  const uint32_t cl = __popc(lo);
  uint32_t up = r >= cl;
  uint32_t w = up ? hi : lo;
  r -= up ? cl : 0u;
  uint32_t pos = up << 5;
  uint32_t c = __popc(w & 0xFFFFu);
  up = r >= c; w = up ? w >> 16 : w; r -= up ? c : 0u; pos += up << 4;
  c = __popc(w & 0xFFu);
  up = r >= c; w = up ? w >> 8 : w; r -= up ? c : 0u; pos += up << 3;
  c = __popc(w & 0xFu);
  up = r >= c; w = up ? w >> 4 : w; r -= up ? c : 0u; pos += up << 2;
  c = __popc(w & 0x3u);
  up = r >= c; w = up ? w >> 2 : w; r -= up ? c : 0u; pos += up << 1;
  c = w & 1u;
  pos += (r >= c) ? 1u : 0u;
  return pos;
}

// position of the i-th (1-based) set bit of x (bits::sel semantics); i <= popc(x)
__device__ __forceinline__ uint32_t sel64(uint64_t x, uint32_t i) { return sel64_0(x, i - 1); }

// d-th (0-based) set bit of v, d < popc(v); cl = popcount of its low 32
// bits.  Halving by popcounts down to a byte, then a 256 x 8 table of
// in-byte selects (lut[byte * 8 + r] = position of the r-th set bit of
// byte), kept in shared memory by the caller (sel_lut_init).
__device__ __forceinline__ uint32_t sel64_lut(uint64_t v, uint32_t d, uint32_t cl, const uint8_t* __restrict__ lut) {
  const bool up = d >= cl;
  uint32_t w = up ? (uint32_t)(v >> 32) : (uint32_t)v;
  d -= up ? cl : 0u;
  uint32_t pos = up ? 32u : 0u;
  const uint32_t c16 = __popc(w & 0xFFFFu);
  const bool u16 = d >= c16;
  w = u16 ? (w >> 16) : w;
  d -= u16 ? c16 : 0u;
  pos += u16 ? 16u : 0u;
  const uint32_t c8 = __popc(w & 0xFFu);
  const bool u8 = d >= c8;
  w = u8 ? (w >> 8) : w;
  d -= u8 ? c8 : 0u;
  pos += u8 ? 8u : 0u;
  return pos + lut[((w & 0xFFu) << 3) | (d & 7u)];
}

// fills the in-byte select table (every thread of the block takes part; a
// barrier must follow before the first use)
__device__ __forceinline__ void sel_lut_init(uint8_t* lut) {
  for (uint32_t e = threadIdx.x; e < 256 * 8; e += blockDim.x) {
    uint32_t byte = e >> 3, r = e & 7, pos = 0;
    for (uint32_t k = 0; k < 8; ++k)
      if ((byte >> k) & 1u) {
        if (r == 0) {
          pos = k;
          break;
        }
        --r;
      }
    lut[e] = (uint8_t)pos;
  }
}

// sdsl bits::hi (0 for x == 0)
__host__ __device__ __forceinline__ uint32_t hi64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return x ? 63u - __clzll((long long)x) : 0u;
#else
  return x ? 63u - (uint32_t)__builtin_clzll(x) : 0u;
#endif
}

// entry j of an int_vector<0> of width w stored at words
__device__ __forceinline__ uint64_t packed_get(const uint64_t* __restrict__ words, uint64_t j, uint32_t w) {
  uint64_t off = j * (uint64_t)w;
  uint64_t wi = off >> 6;
  uint32_t sh = (uint32_t)(off & 63);
  uint64_t v = words[wi] >> sh;
  if (sh + w > 64) v |= words[wi + 1] << (64 - sh);
  return w < 64 ? (v & ((1ull << w) - 1)) : v;
}

// output word q of an int_vector<0> of width w whose entries are given by f(j)
// (entries j >= count are zero); 32-bit offsets while the bit position fits
template <typename F>
__device__ __forceinline__ uint64_t packed_word(uint64_t q, uint32_t w, uint64_t count, F f) {
  const uint64_t mask = w < 64 ? ((1ull << w) - 1) : ~0ull;
  uint64_t out = 0;
  if (q < (1ull << 25)) {  // q*64 + 63 < 2^31
    const uint32_t lo = (uint32_t)q * 64, hi = lo + 63;
    const uint32_t j0 = lo / w, j1 = hi / w;
    for (uint32_t j = j0; j <= j1 && j < count; ++j) {
      const uint64_t v = f((uint64_t)j) & mask;
      const int32_t sh = (int32_t)(j * w) - (int32_t)lo;
      out |= sh >= 0 ? (v << sh) : (v >> (-sh));
    }
    return out;
  }
  const uint64_t lo = q * 64, hi = lo + 63;
  const uint64_t j0 = lo / w, j1 = hi / w;
  for (uint64_t j = j0; j <= j1 && j < count; ++j) {
    const uint64_t v = f(j) & mask;
    const int64_t sh = (int64_t)(j * w) - (int64_t)lo;
    out |= sh >= 0 ? (v << sh) : (v >> (-sh));
  }
  return out;
}

// ------------------------------------------- bulk copies and mbarriers
// 1-D bulk copy global -> shared (cp.async.bulk, completion counted on an
// mbarrier in bytes).  Source and destination 16-byte aligned, size a
// multiple of 16.  Every wait is bounded.

constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 24;
constexpr uint32_t LB_SPIN_LIMIT = 1u << 22;  // ~ seconds with the look-back backoff below

// Limits of the bounded device waits: [0] look-back spins, [1] mbarrier
// tries.  Every translation unit that waits holds its own copy (the library
// is built without relocatable device code); wtg_set_wait_limits rewrites
// them all through the setters declared below, for the current device.
static __constant__ uint32_t c_wait_limit[2] = {LB_SPIN_LIMIT, MBAR_SPIN_LIMIT};
#define WTG_WAIT_LIMIT_SETTER(name)                                                    \
  int set_wait_limits_##name(const uint32_t lim[2]) {                                   \
    cudaError_t e = cudaMemcpyToSymbol(c_wait_limit, lim, 2 * sizeof(uint32_t));        \
    return e == cudaSuccess ? (int)WTG_OK : cuda_fail(e, "cudaMemcpyToSymbol(wait limits)"); \
  }
int set_wait_limits_build(const uint32_t lim[2]);
int set_wait_limits_batch(const uint32_t lim[2]);
int set_wait_limits_bitvec(const uint32_t lim[2]);
int set_wait_limits_core(const uint32_t lim[2]);

// Host-side failure injection for the tests (no device fault is ever made):
// test_take_alloc_failure() is true for the one device allocation the armed
// countdown selects (DevBuf::ensure then reports WTG_ERR_OOM);
// test_take_lookback_stall() is true once after arming, and the rank/select
// pass then starts its tile counter at 1, so tile 0 never publishes and the
// other tiles' bounded look-back waits run out.
bool test_take_alloc_failure();
bool test_take_lookback_stall();
void test_arm_alloc_failure(int64_t nth);
void test_arm_lookback_stall(int on);

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// waits for phase `parity` of bar to complete; false (and err set) on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint32_t limit = c_wait_limit[1];
  for (uint32_t k = 1; k < limit; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  atomicCAS(err, 0u, (uint32_t)DERR_LOOKBACK_TIMEOUT);
  return false;
}

// ------------------------------------------------ decoupled look-back scan
//
// Single-pass scan status words (Merrill & Garland, "Single-pass Parallel
// Prefix Scan with Decoupled Look-back", 2016): each tile publishes its
// aggregate, then its inclusive prefix.  64-bit word = flag (2 bits) | value.
// Tiles take their index from an atomic counter, so every predecessor of a
// tile has already started and the chain always completes; every wait is
// nevertheless bounded, and on expiry the tile records DERR_LOOKBACK_TIMEOUT
// and proceeds (the host then reports the build as failed).

constexpr uint64_t LB_FLAG_AGG = 1ull << 62;
constexpr uint64_t LB_FLAG_INC = 2ull << 62;
constexpr uint64_t LB_VALUE_MASK = (1ull << 62) - 1;

__device__ __forceinline__ void lb_publish(uint64_t* status, uint32_t tile, uint64_t flag, uint64_t v) {
  __threadfence();
  atomicExch((unsigned long long*)&status[tile], (unsigned long long)(flag | (v & LB_VALUE_MASK)));
}

__device__ __forceinline__ uint64_t lb_load(const uint64_t* status, uint64_t idx) {
  return *((volatile const unsigned long long*)&status[idx]);
}

// Warp-cooperative look-back; call with the whole warp.  Returns the exclusive
// prefix of `tile` (tile > 0).
__device__ __forceinline__ uint64_t lb_lookback_warp(uint64_t* status, uint32_t tile, uint32_t* err) {
  const uint32_t lane = threadIdx.x & 31;
  uint64_t prefix = 0;
  int64_t base = (int64_t)tile - 1;
  while (base >= 0) {
    int64_t j = base - lane;
    uint64_t s = 0;
    if (j >= 0) {
      uint32_t spins = 0, ns = 32;
      s = lb_load(status, (uint64_t)j);
      while ((s >> 62) == 0) {
        if (++spins > c_wait_limit[0]) {
          atomicCAS(err, 0u, (uint32_t)DERR_LOOKBACK_TIMEOUT);
          s = LB_FLAG_INC;  // give up: treat as an inclusive zero
          break;
        }
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
        s = lb_load(status, (uint64_t)j);
      }
    } else {
      s = LB_FLAG_INC;  // before tile 0: inclusive zero
    }
    uint32_t inc_mask = __ballot_sync(0xffffffffu, (s >> 62) == 2);
    uint64_t v = s & LB_VALUE_MASK;
    if (inc_mask) {
      uint32_t first = __ffs(inc_mask) - 1;  // nearest inclusive predecessor
      if (lane > first) v = 0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      prefix += v;
      break;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    prefix += v;
    base -= 32;
  }
  return prefix;
}

// ------------------------------------------------ bitvector support build
// Device scalars shared by the bitvector-support build steps.
enum {
  INF_M1 = 0,   // number of ones
  INF_M0,       // number of zeros
  INF_LAST1,    // position of the last one + 1
  INF_LAST0,    // position of the last zero + 1
  INF_NLONG1,   // long superblocks of select1
  INF_NLONG0,
  INF_POOL1,    // pool words of select1
  INF_POOL0,
  INF_N = 16
};

// ------------------------------------------------------- host-side pieces

// Stream-ordered device buffer that keeps its allocation across rebuilds.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need, cudaStream_t s);
  void release(cudaStream_t s);
  template <typename T>
  T* as() const { return (T*)p; }
};

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n, DevBuf& scratch, uint32_t* d_err,
                       cudaStream_t s);
int scan_exclusive_u64(const uint64_t* in, uint64_t* out, uint64_t n, DevBuf& scratch, uint32_t* d_err,
                       cudaStream_t s);

// suffix array (and, when d_bwt is given, the BWT) of a device byte text
// (wtg_sa.cu); n < 2^31; returns after the stream has finished the work;
// rounds (optional) gets the number of doubling rounds
int suffix_array_device(const uint8_t* d_text, uint64_t n, uint32_t* d_sa, uint8_t* d_bwt, int* rounds,
                        cudaStream_t s);

// Flat select_support_mcl on the device.
struct SelectDev {
  uint64_t arg_cnt = 0, nsb = 0, logn = 0, logn4 = 0, has_long = 0, sb_nwords = 0, pool_nwords = 0;
  DevBuf ends;      // superblock end positions (upper-bound sized)
  DevBuf starts;    // superblock start positions (upper-bound sized)
  DevBuf desc;      // per superblock descriptor
  DevBuf sizes;     // per superblock pool words (scan input)
  DevBuf sb_words;  // packed m_superblock
  DevBuf pool;      // packed mini/long blocks
  DevBuf long_list; // superblock ids of long blocks
  DevBuf long_ent;  // 4096 unpacked positions per long block
};

// Rank/select support over one bitvector (caller or tree owned words).
struct BvSupport {
  uint64_t size = 0;
  const uint64_t* words = nullptr;  // device
  uint32_t flags = 0;
  DevBuf rank;       // rank_support_v table
  DevBuf samples;    // every 64th arg, low 32 bits: select1 from the front, select0 from the back
  DevBuf info;       // device scalars (see bitvec.cu)
  DevBuf status;     // look-back status words + tile counter
  DevBuf scan_tmp;
  SelectDev sel[2];  // [t_b]
  cudaEvent_t rank_done = nullptr;  // when set, recorded once the rank table is complete
};

int bv_build(BvSupport& bv, const uint64_t* d_words, uint64_t size, uint32_t flags, uint32_t* d_err,
             cudaStream_t s);
// the same in three steps: allocate and clear, the pass over the bits, and
// the select structures' finishing kernels
int bv_prepare(BvSupport& bv, const uint64_t* d_words, uint64_t size, uint32_t& flags, cudaStream_t s);
int bv_pass(BvSupport& bv, uint32_t* d_err, cudaStream_t s);
int bv_finish(BvSupport& bv, uint32_t* d_err, cudaStream_t s);
// for a wavelet tree's bits with n % 512 == 0: the same structures from the
// level passes' per-chunk zero counts (chunkcnt) and their scans (chunkpre),
// both [L][stride], in three steps: allocate and clear; the pass over levels
// l0..l1-1 (once over all levels, or level by level in order as each level's
// bits and chunk prefixes are final), which extends lvl_zb (L + 1 words, the
// zeros before each level) to l1; the totals and the select finishing kernels
int bv_levels_begin(BvSupport& bv, const uint64_t* d_words, uint64_t n, int L, uint32_t flags, cudaStream_t s);
int bv_levels_pass(BvSupport& bv, uint64_t n, int l0, int l1, const uint32_t* chunkcnt, const uint32_t* chunkpre,
                   uint64_t stride, uint64_t nchunks, uint64_t* lvl_zb, cudaStream_t s);
int bv_levels_end(BvSupport& bv, int L, const uint64_t* lvl_zb, uint32_t* d_err, cudaStream_t s);
void bv_release(BvSupport& bv, cudaStream_t s);

}  // namespace wtg
