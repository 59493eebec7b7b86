// wtg_build.cu -- level-by-level wavelet-tree construction on the GPU.
//
// The reference (wavelet/levelWT/WT.C:86-270) walks the tree node by node:
// at level l every node writes bit (levels-l-1) of its symbols at
// l*n + position and stably partitions them, zeros first, into the next
// level's buffer.  Here a level is one flat pass over the whole sequence:
//
//   * the level-l order is the input stably sorted by the top l bits of each
//     symbol, so node p of level l is the range [C_l(p), C_l(p+1)) of it;
//   * the level's bits are a coalesced map: one __ballot_sync per warp and row
//     yields 32 bits, staged in shared memory and stored as whole words;
//   * the stable partition is a scatter: with Z(i) = number of zeros before
//     position i at this level (one decoupled look-back scan per level) an
//     element of node p with bit 0 goes to  C_l(p) + Z(i) - Zb(p)  and one with
//     bit 1 to  C_l(p) + zeros(p) + (i - Z(i)) - (C_l(p) - Zb(p)), where
//     zeros(p) is the size of p's left child and Zb(p) the zeros of the
//     level's nodes before p; base_kernel / level_table_kernel fold them into
//     two per-node constants.
//
// Node sizes: a pre-pass histograms the top K = min(L, 12) bits in shared
// memory, which gives C and zeros for levels < K.  For deeper levels the pass
// over level l counts, per node of level l+1, the symbols whose next bit is 0
// (the level order keeps each node contiguous, so a warp aggregates a run of
// rows into one atomic per node), and a small table kernel derives level
// l+1's constants before its pass.
//
// Each level pass is a persistent kernel: CTAs take 16 KB tiles from an atomic
// counter and prefetch the next tile with cp.async.bulk into the other half
// of a double buffer while they process the current one.  Per level the
// sequence is read once and written once, plus n/8 bytes of bits.  The node
// table (WT.C:110,156-159,234-257) follows from the per-node starts and zero
// counts alone.
#include <algorithm>

#include "wtg_internal.cuh"
#include "wtg_tree.cuh"

namespace wtg {

constexpr int LV_THREADS = 256;
constexpr int TOP_BITS = 2;  // bits histogrammed by the pre-pass (ballot counted)

template <typename T>
struct LvShape {
  static constexpr int ROWS = 16384 / (LV_THREADS * (int)sizeof(T));  // rows of 32 symbols per warp
  static constexpr uint32_t TILE = LV_THREADS * ROWS;                  // symbols per tile (16 KB)
  static constexpr uint32_t BYTES = TILE * sizeof(T);
  static constexpr int NW = ROWS * (LV_THREADS / 32);  // 32-bit words of level bits per tile
  static constexpr int LOG_TILE = sizeof(T) == 1 ? 14 : sizeof(T) == 2 ? 13 : sizeof(T) == 4 ? 12 : 11;
};

// ------------------------------------------------------------ pre-pass
// One read of the input, tile by tile: the zero count of level 0 in every
// tile (its bit levels-1), and the histogram of the top K <= 2 key bits,
// both counted with warp ballots.

template <typename T>
__global__ void __launch_bounds__(LV_THREADS) prepass_kernel(const T* __restrict__ s, uint64_t n, int L, int K,
                                                             uint32_t* __restrict__ tilecnt,
                                                             uint32_t* __restrict__ hist) {
  using S = LvShape<T>;
  __shared__ uint32_t s_wz[LV_THREADS / 32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t ntiles = (n + S::TILE - 1) / S::TILE;
  uint32_t h[4] = {0, 0, 0, 0};
  const int top = L - 1;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t base = tile * S::TILE + (uint64_t)warp * (S::ROWS * 32);
    uint32_t wz = 0;
#pragma unroll 4
    for (int r = 0; r < S::ROWS; ++r) {
      const uint64_t i = base + r * 32 + lane;
      const bool valid = i < n;
      const uint64_t x = valid ? (uint64_t)s[i] : 0ull;
      const uint32_t b1 = (uint32_t)(x >> top) & 1u;
      const uint32_t b2 = K > 1 ? (uint32_t)(x >> (top - 1)) & 1u : 0u;
      const uint32_t vm = __ballot_sync(0xffffffffu, valid);
      const uint32_t z = __ballot_sync(0xffffffffu, valid && !b1);       // top bits 0x
      const uint32_t z01 = __ballot_sync(0xffffffffu, valid && !b1 && b2);  // 01
      const uint32_t o11 = __ballot_sync(0xffffffffu, valid && b1 && b2);   // 11
      wz += __popc(z);
      h[0] += __popc(z) - __popc(z01);
      h[1] += __popc(z01);
      h[2] += __popc(vm) - __popc(z) - __popc(o11);
      h[3] += __popc(o11);
    }
    if (lane == 0) s_wz[warp] = wz;
    __syncthreads();
    if (tid == 0) {
      uint32_t t = 0;
      for (int w = 0; w < LV_THREADS / 32; ++w) t += s_wz[w];
      tilecnt[tile] = t;
    }
    __syncthreads();
  }
  if (lane == 0) {
    // bins of the top K bits (K = 1: bins 0/1 = top bit 0/1)
    if (K > 1) {
      for (int b = 0; b < 4; ++b)
        if (h[b]) atomicAdd(&hist[b], h[b]);
    } else {
      if (h[0] + h[1]) atomicAdd(&hist[0], h[0] + h[1]);
      if (h[2] + h[3]) atomicAdd(&hist[1], h[2] + h[3]);
    }
  }
}

template <typename T>
__global__ void max_kernel(const T* __restrict__ s, uint64_t n, unsigned long long* out) {
  uint64_t m = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t x = s[i];
    m = x > m ? x : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, (unsigned long long)m);
}

// ------------------------------------------------------ per-node tables
// Heap id h = 2^l - 1 + p names node p of level l (levelWT/WT.C:236-252).
// C[h] = start of node h in its level, Z[h] = size of its left child.

__device__ __forceinline__ void heap_split(uint64_t h, int& l, uint64_t& p) {
  l = 63 - __clzll((long long)(h + 1));
  p = h + 1 - (1ull << l);
}

// levels < K from the top-K histogram scan S (S[2^K] = n)
__global__ void top_tables_kernel(const uint32_t* __restrict__ S, int K, uint32_t* __restrict__ C,
                                  uint32_t* __restrict__ Z) {
  const uint64_t total = (1ull << K) - 1;
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < total;
       h += (uint64_t)gridDim.x * blockDim.x) {
    int l;
    uint64_t p;
    heap_split(h, l, p);
    const uint32_t c = S[p << (K - l)];
    C[h] = c;
    Z[h] = S[(2 * p + 1) << (K - l - 1)] - c;
  }
}

// base(h) = (C - Zb, zeros + Zb) for levels < K; ZS is the exclusive scan of
// Z over heap ids 0..2^K-2 (so Zb = ZS[h] - ZS[first id of h's level])
__global__ void base_kernel(const uint32_t* __restrict__ C, const uint32_t* __restrict__ Z,
                            const uint32_t* __restrict__ ZS, int K, uint2* __restrict__ base) {
  const uint64_t total = (1ull << K) - 1;
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < total;
       h += (uint64_t)gridDim.x * blockDim.x) {
    int l;
    uint64_t p;
    heap_split(h, l, p);
    const uint32_t zb = ZS[h] - ZS[(1ull << l) - 1];
    base[h] = make_uint2(C[h] - zb, Z[h] + zb);
  }
}

// level m >= K: starts from level m-1, and (when m scatters) the constants
// from the level's emitted zero counts and their exclusive scan ZSm
__global__ void level_table_kernel(int m, int with_base, uint32_t* __restrict__ C, const uint32_t* __restrict__ Z,
                                   const uint32_t* __restrict__ ZSm, uint2* __restrict__ base) {
  const uint64_t cnt = 1ull << m;
  const uint64_t first = cnt - 1, pfirst = (cnt >> 1) - 1;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt;
       q += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h = first + q, ph = pfirst + (q >> 1);
    const uint32_t c = C[ph] + ((q & 1) ? Z[ph] : 0u);
    C[h] = c;
    if (with_base) {
      const uint32_t zb = ZSm[q];
      base[h] = make_uint2(c - zb, Z[h] + zb);
    }
  }
}

// WTnode records in heap order (levelWT/WT.C:89-110,156-159,234-257).
__global__ void node_kernel(const uint32_t* __restrict__ C, const uint32_t* __restrict__ Z, int L, uint64_t n,
                            uint64_t n_entries, int ib, void* __restrict__ out) {
  uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= n_entries) return;
  const uint64_t none = ib == 4 ? 0xFFFFFFFFull : ~0ull;
  uint64_t rec[5] = {0, 0, 0, 0, 0};
  if (h == 0) rec[2] = none;
  if (h < (1ull << L) - 1) {
    int l;
    uint64_t p;
    heap_split(h, l, p);
    const uint32_t start = C[h];
    const uint32_t len = (p + 1 < (1ull << l)) ? C[h + 1] - start : (uint32_t)n - start;
    if (h == 0 || len > 0) {
      rec[0] = (uint64_t)l * n + start;
      rec[1] = len;
      rec[2] = h == 0 ? none : (h - 1) / 2;
      if (l < L - 1) {
        const uint32_t z = Z[h];
        rec[3] = z ? 2 * h + 1 : none;
        rec[4] = (len - z) ? 2 * h + 2 : none;
      } else {
        rec[3] = rec[4] = none;
      }
    }
  }
  if (ib == 4) {
    uint32_t* o = (uint32_t*)out + 5 * h;
    for (int k = 0; k < 5; ++k) o[k] = (uint32_t)rec[k];
  } else {
    uint64_t* o = (uint64_t*)out + 5 * h;
    for (int k = 0; k < 5; ++k) o[k] = rec[k];
  }
}

// ------------------------------------------------------------ level pass

// Warp-uniform two-entry counter cache: counts per key are accumulated in
// registers and added to `target` (one atomic) when a key is evicted.  Keys
// of a row arrive sorted by node or by destination, so two entries catch
// almost every repeat.
struct Slot2 {
  uint32_t ka = 0xFFFFFFFFu, ca = 0, kb = 0xFFFFFFFFu, cb = 0;
};

__device__ __forceinline__ void slot2_count(Slot2& s, bool pend, uint32_t key, uint32_t* __restrict__ target,
                                            uint32_t lane) {
  uint32_t rem = __ballot_sync(0xffffffffu, pend);
  while (rem) {
    const uint32_t k0 = __shfl_sync(0xffffffffu, key, __ffs(rem) - 1);
    const uint32_t mk = __ballot_sync(0xffffffffu, pend && key == k0);
    const uint32_t c = __popc(mk);
    rem &= ~mk;
    if (k0 == s.ka) {
      s.ca += c;
    } else if (k0 == s.kb) {
      s.cb += c;
    } else {
      if (lane == 0 && s.ca) atomicAdd(&target[s.ka], s.ca);
      s.ka = s.kb;
      s.ca = s.cb;
      s.kb = k0;
      s.cb = c;
    }
  }
}

__device__ __forceinline__ void slot2_flush(Slot2& s, uint32_t* __restrict__ target, uint32_t lane) {
  if (lane == 0) {
    if (s.ca) atomicAdd(&target[s.ka], s.ca);
    if (s.cb) atomicAdd(&target[s.kb], s.cb);
  }
  s = Slot2();
}

// One level over the level-l order in src:
//   * bits of level `level` (always);
//   * SCATTER: the stable partition of src into dst (the level-(l+1) order).
//     The tile is partitioned locally in shared memory (its zeros, then its
//     ones, each in order) and every run is then stored contiguously; the
//     tile's zeros-before come from tilepre, so tiles never wait on each
//     other;
//   * EMIT_TILES: for every destination tile of the next level, the number of
//     its symbols whose next-level bit is 0 (the next level's tilepre input);
//   * EMIT_NODES: for every node of the next level, its left-child size.
// Tiles are 16 KB; CTAs are persistent (tile = blockIdx.x + k * gridDim.x)
// and prefetch their next tile with cp.async.bulk into the other buffer.
// Warp w owns rows [w*ROWS, (w+1)*ROWS) of 32 consecutive symbols.
template <typename T, bool SCATTER, bool EMIT_NODES, bool EMIT_TILES>
__global__ void __launch_bounds__(LV_THREADS)
    level_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, int L, int level,
                 const uint2* __restrict__ base_lvl, uint32_t* __restrict__ bits32, uint64_t bit_off,
                 const uint32_t* __restrict__ tilepre, uint32_t* __restrict__ tilecnt_next,
                 uint32_t* __restrict__ znext, uint32_t* err, int bulk_ok) {
  using S = LvShape<T>;
  extern __shared__ __align__(128) unsigned char lv_smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_bits[S::NW];
  __shared__ uint32_t s_wz[LV_THREADS / 32];
  T* const buf0 = (T*)lv_smem;
  T* const buf1 = (T*)(lv_smem + S::BYTES);
  T* const stage = (T*)(lv_smem + 2 * S::BYTES);
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t ntiles = (n + S::TILE - 1) / S::TILE;
  const uint64_t nfull = bulk_ok ? n / S::TILE : 0;  // tiles fetched with bulk copies
  const int shift = L - 1 - level;
  const uint32_t pmask = level ? (uint32_t)((1ull << level) - 1) : 0u;
  const uint32_t ltmask = lanemask_lt();

  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_fence_init();
    if (blockIdx.x < nfull) {
      mbar_expect_tx(&mbar[0], S::BYTES);
      bulk_g2s(buf0, src + (uint64_t)blockIdx.x * S::TILE, S::BYTES, &mbar[0]);
    }
  }
  __syncthreads();
  uint32_t phase0 = 0, phase1 = 0;
  int cur = 0;
  uint32_t cache_p = 0xFFFFFFFFu;  // warp-uniform node constants cache
  uint2 cache_b = make_uint2(0, 0);
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t next = tile + gridDim.x;
    if (tid == 0 && next < nfull) {  // prefetch into the other buffer
      fence_proxy_async_smem();
      mbar_expect_tx(&mbar[cur ^ 1], S::BYTES);
      bulk_g2s(cur ? buf0 : buf1, src + next * S::TILE, S::BYTES, &mbar[cur ^ 1]);
    }
    T* const tb = cur ? buf1 : buf0;
    const uint64_t tile_base = tile * S::TILE;
    const uint32_t nvalid = (uint32_t)min((uint64_t)S::TILE, n - tile_base);
    if (tile < nfull) {
      if (cur) {
        mbar_wait(&mbar[1], phase1, err);
        phase1 ^= 1;
      } else {
        mbar_wait(&mbar[0], phase0, err);
        phase0 ^= 1;
      }
    } else {
      for (uint32_t k = tid; k < S::TILE; k += LV_THREADS) tb[k] = k < nvalid ? src[tile_base + k] : T(0);
      __syncthreads();
    }
    const uint32_t wofs = warp * (S::ROWS * 32);

    // 1. level bits, this warp's zero count, next-level node zero counts
    uint32_t wz = 0;
    Slot2 nodes;
#pragma unroll 4
    for (int r = 0; r < S::ROWS; ++r) {
      const uint32_t k = wofs + r * 32 + lane;
      const bool valid = k < nvalid;
      const uint64_t x = (uint64_t)tb[k];
      const bool one = valid && ((x >> shift) & 1);
      const uint32_t ones = __ballot_sync(0xffffffffu, one);
      const uint32_t zeros = __ballot_sync(0xffffffffu, valid && !one);
      if (lane == 0) s_bits[warp * S::ROWS + r] = ones;
      wz += __popc(zeros);
      if (EMIT_NODES) {
        const uint32_t p = level ? ((uint32_t)(x >> (L - level)) & pmask) : 0u;
        const bool zn = valid && !((x >> (shift - 1)) & 1);
        slot2_count(nodes, zn, 2 * p + (one ? 1u : 0u), znext, lane);
      }
    }
    if (EMIT_NODES) slot2_flush(nodes, znext, lane);
    if (lane == 0) s_wz[warp] = wz;
    __syncthreads();

    // 2. store the bits: tile word j covers global bits [g + 32 j, g + 32 j + 32)
    {
      const uint64_t g = bit_off + tile_base;
      const uint32_t g0 = (uint32_t)(g & 31);
      const uint64_t G = g >> 5;
      for (int j = tid; j <= S::NW; j += LV_THREADS) {
        if (g0 == 0 && j == S::NW) break;
        const uint32_t curw = j < S::NW ? s_bits[j] : 0u;
        const uint32_t prev = j > 0 ? s_bits[j - 1] : 0u;
        const uint32_t val = g0 ? ((curw << g0) | (prev >> (32 - g0))) : curw;
        const uint64_t wlo = (G + j) * 32;
        if (wlo >= g + nvalid) continue;
        const bool full = (wlo >= g) && (wlo + 32 <= g + nvalid);
        if (full) bits32[G + j] = val;
        else if (val) atomicOr(&bits32[G + j], val);
      }
    }

    if (SCATTER) {
      // 3. local stable partition: zeros of the tile first, then its ones
      uint32_t zt = 0, zl = 0;
#pragma unroll
      for (uint32_t w = 0; w < LV_THREADS / 32; ++w) {
        const uint32_t c = s_wz[w];
        zl += w < warp ? c : 0u;
        zt += c;
      }
#pragma unroll 4
      for (int r = 0; r < S::ROWS; ++r) {
        const uint32_t k = wofs + r * 32 + lane;
        const bool valid = k < nvalid;
        const T x = tb[k];
        const bool one = valid && (((uint64_t)x >> shift) & 1);
        const uint32_t zm = __ballot_sync(0xffffffffu, valid && !one);
        const uint32_t zb = zl + __popc(zm & ltmask);
        zl += __popc(zm);
        if (valid) stage[one ? zt + (k - zb) : zb] = x;
      }
      __syncthreads();

      // 4. store the runs: slot j < zt is the tile's j-th zero, slot j >= zt
      //    its (j - zt)-th one; consecutive slots of a node go to consecutive
      //    destinations
      const uint32_t zpre = tilepre[tile];
      const uint32_t opre = (uint32_t)tile_base - zpre;
      Slot2 tiles;
      for (uint32_t j0 = warp * 32; j0 < nvalid; j0 += LV_THREADS) {
        const uint32_t j = j0 + lane;
        const bool valid = j < nvalid;
        const T x = stage[valid ? j : j0];
        const uint32_t p = level ? ((uint32_t)((uint64_t)x >> (L - level)) & pmask) : 0u;
        const uint32_t p0 = __shfl_sync(0xffffffffu, p, 0);
        uint2 b;
        if (__ballot_sync(0xffffffffu, valid && p != p0) == 0) {
          if (p0 != cache_p) {
            cache_p = p0;
            cache_b = base_lvl[p0];
          }
          b = cache_b;
        } else {
          b = base_lvl[p];
        }
        const uint32_t d = j >= zt ? b.y + opre + (j - zt) : b.x + zpre + j;
        const bool ok = valid && d < n;
        if (ok) dst[d] = x;
        else if (valid) atomicCAS(err, 0u, (uint32_t)DERR_BAD_INDEX);
        if (EMIT_TILES) {
          const bool pend = ok && !(((uint64_t)x >> (shift - 1)) & 1);
          slot2_count(tiles, pend, d >> S::LOG_TILE, tilecnt_next, lane);
        }
      }
      if (EMIT_TILES) slot2_flush(tiles, tilecnt_next, lane);
    }
    __syncthreads();
    cur ^= 1;
  }
}

// ------------------------------------------------------------------ host

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <typename T>
static void launch_max(const void* s, uint64_t n, unsigned long long* out, cudaStream_t st) {
  unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8);
  if (grid == 0) grid = 1;
  max_kernel<T><<<grid, 256, 0, st>>>((const T*)s, n, out);
}

template <typename T, bool SC, bool EN, bool ET>
static int level_grid(uint64_t n) {
  static int per_sm = 0;
  if (!per_sm) {
    cudaFuncSetAttribute(level_kernel<T, SC, EN, ET>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(level_kernel<T, SC, EN, ET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(3 * LvShape<T>::BYTES));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, level_kernel<T, SC, EN, ET>, LV_THREADS,
                                                  3 * LvShape<T>::BYTES);
    if (per_sm <= 0) per_sm = 1;
  }
  const uint64_t tiles = (n + LvShape<T>::TILE - 1) / LvShape<T>::TILE;
  return (int)std::min<uint64_t>(tiles, (uint64_t)per_sm * sm_count());
}

template <typename T>
static void launch_level(const void* src, void* dst, uint64_t n, int L, int level, const uint2* base_lvl,
                         uint32_t* bits32, uint64_t bit_off, const uint32_t* tilepre, uint32_t* tilecnt_next,
                         uint32_t* znext, uint32_t* err, bool scatter, bool emit_nodes, bool emit_tiles,
                         cudaStream_t st) {
  const int bulk_ok = ((uintptr_t)src % 16) == 0;
  const size_t shm = 3 * LvShape<T>::BYTES;
#define WTG_LV(SC, EN, ET)                                                                                \
  level_kernel<T, SC, EN, ET><<<level_grid<T, SC, EN, ET>(n), LV_THREADS, shm, st>>>(                    \
      (const T*)src, (T*)dst, n, L, level, base_lvl, bits32, bit_off, tilepre, tilecnt_next, znext, err, \
      bulk_ok)
  if (scatter && emit_nodes) WTG_LV(true, true, true);
  else if (scatter && emit_tiles) WTG_LV(true, false, true);
  else if (scatter) WTG_LV(true, false, false);
  else WTG_LV(false, false, false);
#undef WTG_LV
}

template <typename T>
static void launch_prepass(const void* s, uint64_t n, int L, int K, uint32_t* tilecnt, uint32_t* hist,
                           cudaStream_t st) {
  const uint64_t tiles = (n + LvShape<T>::TILE - 1) / LvShape<T>::TILE;
  unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sm_count() * 8);
  if (grid == 0) grid = 1;
  prepass_kernel<T><<<grid, LV_THREADS, 0, st>>>((const T*)s, n, L, K, tilecnt, hist);
}

#define WTG_DISPATCH(eb, fn, ...)                       \
  switch (eb) {                                         \
    case 1: fn<uint8_t>(__VA_ARGS__); break;            \
    case 2: fn<uint16_t>(__VA_ARGS__); break;           \
    case 4: fn<uint32_t>(__VA_ARGS__); break;           \
    default: fn<uint64_t>(__VA_ARGS__); break;          \
  }

static uint64_t tile_elems(int eb) { return 16384 / eb; }

int tree_levels_from_max(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int* levels) {
  cudaStream_t s = t.stream;
  int rc;
  if ((rc = t.scratch.ensure(sizeof(unsigned long long), s))) return rc;
  WTG_CK(cudaMemsetAsync(t.scratch.p, 0, sizeof(unsigned long long), s));
  if (n) {
    WTG_DISPATCH(eb, launch_max, d_seq, n, t.scratch.as<unsigned long long>(), s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  unsigned long long mx = 0;
  WTG_CK(cudaMemcpyAsync(&mx, t.scratch.p, sizeof(mx), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  if (mx < 1) mx = 1;
  *levels = (int)hi64(mx) + 1;  // wt_int_par.hpp:385-395 (x starts at 1)
  return WTG_OK;
}

int tree_build(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int L, uint32_t flags) {
  cudaStream_t s = t.stream;
  int rc;
  t.n = n;
  t.levels = L;
  t.elem_bytes = eb;
  t.flags = flags;
  t.bit_words = (n * (uint64_t)L + 63) / 64;
  const int K = std::min(L, TOP_BITS);
  const uint64_t heap = 1ull << L;  // heap ids 0 .. 2^L - 2, plus one pad entry

  if ((rc = t.err.ensure(sizeof(uint32_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(t.err.p, 0, sizeof(uint32_t), s));
  uint32_t* d_err = t.err.as<uint32_t>();

  if ((rc = t.bits.ensure((t.bit_words + 2) * sizeof(uint64_t), s))) return rc;
  if (n % 32 != 0 || n == 0) {
    WTG_CK(cudaMemsetAsync(t.bits.p, 0, (t.bit_words + 2) * sizeof(uint64_t), s));
  } else {
    // every 32-bit word of level data is stored whole; clear the last data
    // word (its high half may lie past n*L) and the trailing zero word
    uint64_t from = t.bit_words ? t.bit_words - 1 : 0;
    WTG_CK(cudaMemsetAsync(t.bits.as<uint64_t>() + from, 0, (t.bit_words + 2 - from) * sizeof(uint64_t), s));
  }

  // per-node tables: hist = top-K histogram scan; zeros = [Z | ZS | C]
  if ((rc = t.hist.ensure(((1ull << K) + 1) * sizeof(uint32_t), s))) return rc;
  if ((rc = t.zeros.ensure(3 * heap * sizeof(uint32_t), s))) return rc;
  if ((rc = t.base.ensure(heap * sizeof(uint2), s))) return rc;
  uint32_t* S = t.hist.as<uint32_t>();
  uint32_t* Z = t.zeros.as<uint32_t>();
  uint32_t* ZS = Z + heap;
  uint32_t* C = Z + 2 * heap;
  uint2* base = t.base.as<uint2>();
  WTG_CK(cudaMemsetAsync(S, 0, ((1ull << K) + 1) * sizeof(uint32_t), s));
  WTG_CK(cudaMemsetAsync(Z, 0, 3 * heap * sizeof(uint32_t), s));

  // per-level tile zero counts [L x tiles] and their scan (tilepre)
  const uint64_t tiles = n ? (n + tile_elems(eb) - 1) / tile_elems(eb) : 0;
  if ((rc = t.status.ensure(((uint64_t)L + 1) * (tiles + 1) * sizeof(uint32_t), s))) return rc;
  uint32_t* tilecnt = t.status.as<uint32_t>();
  uint32_t* tilepre = tilecnt + (uint64_t)L * (tiles + 1);
  if (n) WTG_CK(cudaMemsetAsync(tilecnt, 0, (uint64_t)L * (tiles + 1) * sizeof(uint32_t), s));

  if (n) {
    prof_begin(PROF_HIST, s);
    WTG_DISPATCH(eb, launch_prepass, d_seq, n, L, K, tilecnt, S, s);
    prof_end(PROF_HIST, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  if ((rc = scan_exclusive_u32(S, S, (1ull << K) + 1, t.scan_tmp, d_err, s))) return rc;
  {
    const uint64_t top = (1ull << K) - 1;
    prof_begin(PROF_TABLES, s);
    top_tables_kernel<<<1, 256, 0, s>>>(S, K, C, Z);
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = scan_exclusive_u32(Z, ZS, top + 1, t.scan_tmp, d_err, s))) return rc;
    prof_begin(PROF_TABLES, s);
    base_kernel<<<1, 256, 0, s>>>(C, Z, ZS, K, base);
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }

  // level passes; each scattering pass feeds the next level's tile counts
  // and (from level K on) its node tables
  if (n) {
    if (L > 1) {
      if ((rc = t.lvl[0].ensure(n * eb + 16, s))) return rc;
      if ((rc = t.lvl[1].ensure(n * eb + 16, s))) return rc;
    }
    const void* src = d_seq;
    for (int l = 0; l < L; ++l) {
      const bool scatter = l < L - 1;
      const bool emit_tiles = l + 1 <= L - 2;
      const bool emit_nodes = emit_tiles && (l + 1 >= K);
      void* dst = scatter ? t.lvl[l & 1].p : nullptr;
      if (scatter)
        if ((rc = scan_exclusive_u32(tilecnt + (uint64_t)l * (tiles + 1), tilepre, tiles, t.scan_tmp, d_err, s)))
          return rc;
      uint32_t* znext = Z + ((1ull << (l + 1)) - 1);
      uint32_t* tnext = tilecnt + (uint64_t)(l + 1) * (tiles + 1);
      prof_begin(scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      WTG_DISPATCH(eb, launch_level, src, dst, n, L, l, base + ((1ull << l) - 1), t.bits.as<uint32_t>(),
                   (uint64_t)l * n, tilepre, tnext, znext, d_err, scatter, emit_nodes, emit_tiles, s);
      prof_end(scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      count_launch();
      WTG_CK(cudaGetLastError());
      src = dst;
      const int m = l + 1;  // next level: derive its tables when the pre-pass did not
      if (m >= K && m <= L - 1) {
        const uint64_t cnt = 1ull << m;
        const int with_base = m <= L - 2;
        if (with_base)
          if ((rc = scan_exclusive_u32(Z + cnt - 1, ZS, cnt, t.scan_tmp, d_err, s))) return rc;
        unsigned grid = (unsigned)std::min<uint64_t>((cnt + 255) / 256, 2048);
        prof_begin(PROF_TABLES, s);
        level_table_kernel<<<grid, 256, 0, s>>>(m, with_base, C, Z, ZS, base);
        prof_end(PROF_TABLES, s);
        count_launch();
        WTG_CK(cudaGetLastError());
      }
    }
  }

  // rank / select over the concatenated bitvector
  if (flags) {
    if ((rc = bv_build(t.bv, t.bits.as<uint64_t>(), n * (uint64_t)L, flags, d_err, s))) return rc;
  }
  return WTG_OK;
}

int tree_nodes(TreeImpl& t, int ib, uint64_t n_entries, void* d_out) {
  cudaStream_t s = t.stream;
  if (n_entries == 0) return WTG_OK;
  const uint64_t heap = 1ull << t.levels;
  uint32_t* Z = t.zeros.as<uint32_t>();
  unsigned grid = (unsigned)((n_entries + 255) / 256);
  node_kernel<<<grid, 256, 0, s>>>(Z + 2 * heap, Z, t.levels, t.n, n_entries, ib, d_out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

void tree_release(TreeImpl& t) {
  cudaStream_t s = t.stream;
  t.seq.release(s);
  t.lvl[0].release(s);
  t.lvl[1].release(s);
  t.bits.release(s);
  t.hist.release(s);
  t.zeros.release(s);
  t.base.release(s);
  t.status.release(s);
  t.scan_tmp.release(s);
  t.err.release(s);
  t.scratch.release(s);
  t.nodes.release(s);
  bv_release(t.bv, s);
}

}  // namespace wtg
