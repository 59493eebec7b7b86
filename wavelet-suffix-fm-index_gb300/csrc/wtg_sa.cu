// wtg_sa.cu -- suffix array and BWT of a byte text on the GPU: the first two
// steps of the reference's FM-index construction (fm-index/par/WT.C:33-41:
// divsufsort, then bwt[i] = s[SA[i] - 1], or s[n - 1] where SA[i] = 0).
//
// Prefix doubling (Manber & Myers, "Suffix arrays: a new method for on-line
// string searches", 1993) over LSD radix sorts:
//   * the text's distinct bytes get codes 1..sigma (0 = past the end), b bits
//     each; a suffix's first K = floor(64 / b) characters, packed
//     most-significant first, are its initial 64-bit key, so key order is the
//     order of the K-character prefixes (a prefix cut by the end sorts first);
//   * after a sort, rank[i] = the suffix-array position of the first slot of
//     suffix i's group (suffixes with equal keys); while groups of several
//     suffixes remain, only their members are re-keyed by
//     (rank[i], rank[i + h] + 1 or 0 past the end) and re-sorted, and h
//     doubles (finished groups are never touched again).
// The sort is stable and every rank is a function of the key, so the result
// is the unique suffix order, the same array divsufsort gives.
#include <algorithm>
#include <vector>

#include "wtg_internal.cuh"

namespace wtg {

namespace {

constexpr int SA_THREADS = 256;
constexpr int SA_WARPS = SA_THREADS / 32;
constexpr int SA_IPW = 512;                    // elements per warp and tile
constexpr int SA_TILE = SA_WARPS * SA_IPW;     // elements per tile (4096)
constexpr int RBITS = 8;                       // radix digit
constexpr int RADIX = 1 << RBITS;

__global__ void byte_hist_kernel(const uint8_t* __restrict__ s, uint64_t n, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[SA_WARPS][256];
  for (uint32_t i = threadIdx.x; i < SA_WARPS * 256; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  const uint32_t w = threadIdx.x >> 5;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[w][s[i]], 1u);
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x) {
    uint32_t t = 0;
    for (int k = 0; k < SA_WARPS; ++k) t += h[k][c];
    if (t) atomicAdd(&hist[c], t);
  }
}

// key[i] = codes of s[i .. i + K) packed from the top (0 past the end)
__global__ void init_keys_kernel(const uint8_t* __restrict__ s, uint64_t n, const uint16_t* __restrict__ code_g,
                                 int b, int K, uint64_t* __restrict__ key, uint32_t* __restrict__ val) {
  __shared__ uint16_t code[256];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) code[i] = code_g[i];
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t k = 0;
    for (int c = 0; c < K; ++c) {
      const uint64_t x = i + c < n ? code[s[i + c]] : 0u;
      k |= x << (64 - b * (c + 1));
    }
    key[i] = k;
    val[i] = (uint32_t)i;
  }
}

// per tile, its count of every digit: counts[digit * ntiles + tile]
__global__ void __launch_bounds__(SA_THREADS) radix_count_kernel(const uint64_t* __restrict__ key, uint64_t n,
                                                                int shift, uint32_t* __restrict__ counts,
                                                                uint32_t ntiles) {
  __shared__ uint32_t h[SA_WARPS][RADIX];
  for (uint32_t i = threadIdx.x; i < SA_WARPS * RADIX; i += SA_THREADS) (&h[0][0])[i] = 0;
  __syncthreads();
  const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t base = (uint64_t)blockIdx.x * SA_TILE + (uint64_t)w * SA_IPW;
  for (int it = 0; it < SA_IPW / 32; ++it) {
    const uint64_t idx = base + it * 32 + lane;
    if (idx < n) atomicAdd(&h[w][(uint32_t)(key[idx] >> shift) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < RADIX; d += SA_THREADS) {
    uint32_t t = 0;
    for (int k = 0; k < SA_WARPS; ++k) t += h[k][d];
    counts[(uint64_t)d * ntiles + blockIdx.x] = t;
  }
}

// stable scatter of one tile: offs = exclusive scan of counts.  A warp ranks
// its 512 elements in order (equal digits of one step ranked by lane) into a
// digit-sorted copy of the tile in shared memory; the block then writes the
// copy out in order, so each digit's run goes out as consecutive stores.
__global__ void __launch_bounds__(SA_THREADS) radix_scatter_kernel(const uint64_t* __restrict__ key,
                                                                  const uint32_t* __restrict__ val, uint64_t n,
                                                                  int shift, const uint32_t* __restrict__ offs,
                                                                  uint32_t ntiles, uint64_t* __restrict__ key_out,
                                                                  uint32_t* __restrict__ val_out) {
  extern __shared__ __align__(16) unsigned char sa_smem[];
  uint64_t* const skey = (uint64_t*)sa_smem;                  // SA_TILE keys
  uint32_t* const sval = (uint32_t*)(skey + SA_TILE);         // SA_TILE values
  __shared__ uint32_t wc[SA_WARPS][RADIX];                    // per warp: count, then local base
  __shared__ int64_t gdelta[RADIX];                           // global position - local index
  __shared__ uint32_t wsum[SA_WARPS];
  for (uint32_t i = threadIdx.x; i < SA_WARPS * RADIX; i += SA_THREADS) (&wc[0][0])[i] = 0;
  __syncthreads();
  const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const uint64_t tile0 = (uint64_t)blockIdx.x * SA_TILE;
  const uint32_t tn = (uint32_t)min((uint64_t)SA_TILE, n - tile0);  // elements in this tile
  const uint64_t base = tile0 + (uint64_t)w * SA_IPW;
  for (int it = 0; it < SA_IPW / 32; ++it) {
    const uint64_t idx = base + it * 32 + lane;
    const bool valid = idx < n;
    const uint32_t d = valid ? (uint32_t)(key[idx] >> shift) & (RADIX - 1) : 0xFFFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    if (valid && lane == (uint32_t)(__ffs(peers) - 1)) wc[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // thread d: the tile's count of digit d, its exclusive scan over digits
  // (the digit's first local index) and each warp's local base
  const uint32_t d = threadIdx.x;  // SA_THREADS == RADIX
  uint32_t tot = 0;
  for (int k = 0; k < SA_WARPS; ++k) tot += wc[k][d];
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t q = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += q;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  uint32_t start = inc - tot;
  for (uint32_t k = 0; k < w; ++k) start += wsum[k];
  gdelta[d] = (int64_t)offs[(uint64_t)d * ntiles + blockIdx.x] - (int64_t)start;
  uint32_t run = start;
  for (int k = 0; k < SA_WARPS; ++k) {
    const uint32_t c = wc[k][d];
    wc[k][d] = run;
    run += c;
  }
  __syncthreads();
  for (int it = 0; it < SA_IPW / 32; ++it) {
    const uint64_t idx = base + it * 32 + lane;
    const bool valid = idx < n;
    uint64_t k = 0;
    uint32_t v = 0, dg = 0xFFFFu;
    if (valid) {
      k = key[idx];
      v = val[idx];
      dg = (uint32_t)(k >> shift) & (RADIX - 1);
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, dg);
    if (valid) {
      const uint32_t lp = wc[w][dg] + __popc(peers & lt);
      skey[lp] = k;
      sval[lp] = v;
    }
    __syncwarp();
    if (valid && lane == (uint32_t)(__ffs(peers) - 1)) wc[w][dg] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < tn; j += SA_THREADS) {
    const uint64_t k = skey[j];
    const uint64_t g = (uint64_t)((int64_t)j + gdelta[(uint32_t)(k >> shift) & (RADIX - 1)]);
    key_out[g] = k;
    val_out[g] = sval[j];
  }
}

// Doubling rounds work on the active list: the suffix-array positions
// act[0..m) (ascending) of the suffixes whose group still holds more than
// one suffix.  A group occupies consecutive positions, its members share
// rank = the position of the group's first slot, and sorting the active
// suffixes by (rank, rank of the suffix h on) lays the groups out in
// position order again, so the k-th sorted suffix goes to position act[k].

__device__ __forceinline__ bool run_start(const uint64_t* __restrict__ key, uint64_t k) {
  return k == 0 || key[k] != key[k - 1];
}

// key of active suffix k: the first K codes (round 0, suffix k, act is the
// identity) or (rank[i], rank[i + h] + 1, or 0 past the end) for i = sa[act[k]]
__global__ void active_keys_kernel(const uint32_t* __restrict__ act, const uint32_t* __restrict__ sa,
                                   const uint32_t* __restrict__ rank, uint64_t m, uint64_t n, uint64_t h, int B,
                                   uint64_t* __restrict__ key, uint32_t* __restrict__ val) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = sa[act[k]];
    const uint64_t sec = i + h < n ? (uint64_t)rank[i + h] + 1 : 0;
    key[k] = ((uint64_t)rank[i] << B) | sec;
    val[k] = i;
  }
}

// g[k] = 1 where sorted key k starts a run of equal keys; g[m] = 0
__global__ void run_flags_kernel(const uint64_t* __restrict__ key, uint64_t m, uint32_t* __restrict__ g) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= m; k += (uint64_t)gridDim.x * blockDim.x)
    g[k] = k < m && run_start(key, k) ? 1u : 0u;
}

// after the scan of the run flags: first[r] = sorted index of run r's first key
__global__ void run_first_kernel(const uint64_t* __restrict__ key, const uint32_t* __restrict__ g, uint64_t m,
                                 uint32_t* __restrict__ first) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x)
    if (run_start(key, k)) first[g[k]] = (uint32_t)k;
}

// place the sorted active suffixes, give each the position of its new
// group's first slot as rank, and flag the ones still sharing a group
// (ga[k] = 1, ga[m] = 0, for the scan that compacts the next active list)
__global__ void place_kernel(const uint64_t* __restrict__ key, const uint32_t* __restrict__ val,
                             const uint32_t* __restrict__ g, const uint32_t* __restrict__ first,
                             const uint32_t* __restrict__ act, uint64_t m, uint32_t* __restrict__ sa,
                             uint32_t* __restrict__ rank, uint32_t* __restrict__ ga) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= m; k += (uint64_t)gridDim.x * blockDim.x) {
    if (k == m) {
      ga[m] = 0;
      continue;
    }
    const bool st = run_start(key, k);
    const bool next_st = k + 1 == m || key[k + 1] != key[k];
    const uint32_t i = val[k];
    sa[act[k]] = i;
    rank[i] = act[first[g[k] + (st ? 1u : 0u) - 1u]];
    ga[k] = (st && next_st) ? 0u : 1u;
  }
}

// next active list: act_next[ga[k]] = act[k] for the suffixes still shared
__global__ void compact_active_kernel(const uint64_t* __restrict__ key, const uint32_t* __restrict__ ga,
                                      const uint32_t* __restrict__ act, uint64_t m, uint32_t* __restrict__ act_next) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
    const bool st = run_start(key, k);
    const bool next_st = k + 1 == m || key[k + 1] != key[k];
    if (!(st && next_st)) act_next[ga[k]] = act[k];
  }
}

__global__ void iota_kernel(uint32_t* __restrict__ a, uint64_t m) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x)
    a[k] = (uint32_t)k;
}

// fm-index/par/WT.C:38-41: bwt[j] = s[SA[j] - 1], or s[n - 1] where SA[j] = 0
__global__ void bwt_kernel(const uint8_t* __restrict__ s, const uint32_t* __restrict__ sa, uint64_t n,
                           uint8_t* __restrict__ bwt) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = sa[j];
    bwt[j] = s[p ? p - 1 : n - 1];
  }
}

int bit_width64(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }

unsigned grid_for(uint64_t n) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 16));
}

}  // namespace

// Scratch of one suffix-array run, released when it ends.
struct SaScratch {
  DevBuf key[2], val[2], rank, sa, act[2], g, first, counts, scan_tmp, err, small;
  cudaStream_t s;
  explicit SaScratch(cudaStream_t st) : s(st) {}
  ~SaScratch() {
    for (auto* b : {&key[0], &key[1], &val[0], &val[1], &rank, &sa, &act[0], &act[1], &g, &first, &counts,
                    &scan_tmp, &err, &small})
      b->release(s);
  }
};

// LSD radix sort of (key, val) pairs on key bits [lo, hi); the result is in
// key[cur] / val[cur] (cur flips once per pass)
constexpr int SCATTER_SMEM = SA_TILE * (8 + 4);  // the tile's keys and values

static int radix_sort(SaScratch& x, uint64_t n, int lo, int hi, int& cur) {
  int rc;
  static bool attr = false;
  if (!attr) {
    WTG_CK(cudaFuncSetAttribute(radix_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SCATTER_SMEM));
    attr = true;
  }
  const uint32_t ntiles = (uint32_t)((n + SA_TILE - 1) / SA_TILE);
  for (int shift = lo; shift < hi; shift += RBITS) {
    radix_count_kernel<<<ntiles, SA_THREADS, 0, x.s>>>(x.key[cur].as<uint64_t>(), n, shift, x.counts.as<uint32_t>(),
                                                       ntiles);
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = scan_exclusive_u32(x.counts.as<uint32_t>(), x.counts.as<uint32_t>(), (uint64_t)RADIX * ntiles,
                                 x.scan_tmp, x.err.as<uint32_t>(), x.s)))
      return rc;
    radix_scatter_kernel<<<ntiles, SA_THREADS, SCATTER_SMEM, x.s>>>(x.key[cur].as<uint64_t>(), x.val[cur].as<uint32_t>(), n,
                                                         shift, x.counts.as<uint32_t>(), ntiles,
                                                         x.key[cur ^ 1].as<uint64_t>(), x.val[cur ^ 1].as<uint32_t>());
    count_launch();
    WTG_CK(cudaGetLastError());
    cur ^= 1;
  }
  return WTG_OK;
}

static int scan_u32(SaScratch& x, uint32_t* a, uint64_t m, uint32_t* total) {
  int rc;
  if ((rc = scan_exclusive_u32(a, a, m + 1, x.scan_tmp, x.err.as<uint32_t>(), x.s))) return rc;
  WTG_CK(cudaMemcpyAsync(total, a + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, x.s));
  WTG_CK(cudaStreamSynchronize(x.s));
  uint32_t e = 0;
  WTG_CK(cudaMemcpy(&e, x.err.p, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return fail(WTG_ERR_TIMEOUT, "suffix array: a scan wait timed out");
  return WTG_OK;
}

// after a sort of the m active pairs (in key[cur] / val[cur]): place them,
// refresh their ranks and compact the still-shared ones into act[ac ^ 1]
static int settle_round(SaScratch& x, uint64_t m, int cur, int& ac, uint64_t* m_next) {
  int rc;
  const unsigned grid = grid_for(m + 1);
  const uint64_t* key = x.key[cur].as<uint64_t>();
  uint32_t* g = x.g.as<uint32_t>();
  run_flags_kernel<<<grid, 256, 0, x.s>>>(key, m, g);
  count_launch();
  WTG_CK(cudaGetLastError());
  uint32_t runs = 0;
  if ((rc = scan_u32(x, g, m, &runs))) return rc;
  run_first_kernel<<<grid, 256, 0, x.s>>>(key, g, m, x.first.as<uint32_t>());
  count_launch();
  WTG_CK(cudaGetLastError());
  uint32_t* ga = x.key[cur ^ 1].as<uint32_t>();  // the other key buffer is free until the next sort
  place_kernel<<<grid, 256, 0, x.s>>>(key, x.val[cur].as<uint32_t>(), g, x.first.as<uint32_t>(),
                                      x.act[ac].as<uint32_t>(), m, x.sa.as<uint32_t>(), x.rank.as<uint32_t>(), ga);
  count_launch();
  WTG_CK(cudaGetLastError());
  uint32_t still = 0;
  if ((rc = scan_u32(x, ga, m, &still))) return rc;
  if (still) {
    compact_active_kernel<<<grid, 256, 0, x.s>>>(key, ga, x.act[ac].as<uint32_t>(), m, x.act[ac ^ 1].as<uint32_t>());
    count_launch();
    WTG_CK(cudaGetLastError());
    ac ^= 1;
  }
  *m_next = still;
  return WTG_OK;
}

int suffix_array_device(const uint8_t* d_text, uint64_t n, uint32_t* d_sa, uint8_t* d_bwt, int* rounds,
                        cudaStream_t s) {
  int rc;
  if (rounds) *rounds = 0;
  if (n == 0) return WTG_OK;
  if (n >= (1ull << 31)) return fail(WTG_ERR_INVALID, "suffix array: n must be below 2^31 (32-bit entries)");
  SaScratch x(s);
  const uint64_t ntiles = (n + SA_TILE - 1) / SA_TILE;
  if ((rc = x.key[0].ensure(n * 8 + 8, s)) || (rc = x.key[1].ensure(n * 8 + 8, s)) ||
      (rc = x.val[0].ensure(n * 4, s)) || (rc = x.val[1].ensure(n * 4, s)) || (rc = x.rank.ensure(n * 4, s)) ||
      (rc = x.sa.ensure(n * 4, s)) || (rc = x.act[0].ensure(n * 4, s)) || (rc = x.act[1].ensure(n * 4, s)) ||
      (rc = x.g.ensure((n + 1) * 4, s)) || (rc = x.first.ensure(n * 4, s)) ||
      (rc = x.counts.ensure(RADIX * ntiles * 4, s)) || (rc = x.err.ensure(4, s)) || (rc = x.small.ensure(2048, s)))
    return rc;
  WTG_CK(cudaMemsetAsync(x.err.p, 0, 4, s));
  // alphabet: codes 1..sigma in byte order
  uint32_t* d_hist = x.small.as<uint32_t>();
  WTG_CK(cudaMemsetAsync(d_hist, 0, 256 * 4, s));
  byte_hist_kernel<<<grid_for(n), 256, 0, s>>>(d_text, n, d_hist);
  count_launch();
  WTG_CK(cudaGetLastError());
  uint32_t hist[256];
  WTG_CK(cudaMemcpyAsync(hist, d_hist, sizeof(hist), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  uint16_t code[256];  // 1..sigma, sigma <= 256
  int sigma = 0;
  for (int c = 0; c < 256; ++c) code[c] = hist[c] ? (uint16_t)++sigma : 0;
  const int b = bit_width64((uint64_t)sigma);  // codes 0..sigma
  const int K = 64 / b;
  uint16_t* d_code = (uint16_t*)(x.small.as<uint32_t>() + 256);
  WTG_CK(cudaMemcpyAsync(d_code, code, sizeof(code), cudaMemcpyHostToDevice, s));
  // round 0: every suffix, keyed by its first K codes
  init_keys_kernel<<<grid_for(n), 256, 0, s>>>(d_text, n, d_code, b, K, x.key[0].as<uint64_t>(),
                                               x.val[0].as<uint32_t>());
  count_launch();
  iota_kernel<<<grid_for(n), 256, 0, s>>>(x.act[0].as<uint32_t>(), n);
  count_launch();
  WTG_CK(cudaGetLastError());
  int cur = 0, ac = 0;
  if ((rc = radix_sort(x, n, (64 - b * K) / RBITS * RBITS, 64, cur))) return rc;
  uint64_t m = 0;
  if ((rc = settle_round(x, n, cur, ac, &m))) return rc;
  uint64_t h = (uint64_t)K;
  int r = 0;
  const int B = bit_width64(n);               // rank[i + h] + 1 <= n
  const int hi = B + bit_width64(n - 1);      // rank < n
  while (m) {
    active_keys_kernel<<<grid_for(m), 256, 0, s>>>(x.act[ac].as<uint32_t>(), x.sa.as<uint32_t>(),
                                                   x.rank.as<uint32_t>(), m, n, h, B, x.key[cur].as<uint64_t>(),
                                                   x.val[cur].as<uint32_t>());
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = radix_sort(x, m, 0, hi, cur))) return rc;
    if ((rc = settle_round(x, m, cur, ac, &m))) return rc;
    h *= 2;
    ++r;
  }
  if (rounds) *rounds = r;
  if (d_sa) WTG_CK(cudaMemcpyAsync(d_sa, x.sa.p, n * 4, cudaMemcpyDeviceToDevice, s));
  if (d_bwt) {
    bwt_kernel<<<grid_for(n), 256, 0, s>>>(d_text, x.sa.as<uint32_t>(), n, d_bwt);
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  WTG_CK(cudaStreamSynchronize(s));
  return WTG_OK;
}

}  // namespace wtg
