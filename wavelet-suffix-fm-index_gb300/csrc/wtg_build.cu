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
constexpr int TOP_BITS = 12;  // bits histogrammed by the pre-pass

template <typename T>
struct LvShape {
  static constexpr int ROWS = 16384 / (LV_THREADS * (int)sizeof(T));  // rows of 256 symbols per tile
  static constexpr uint32_t TILE = LV_THREADS * ROWS;                  // symbols per tile (16 KB)
  static constexpr uint32_t BYTES = TILE * sizeof(T);
  static constexpr int NW = ROWS * (LV_THREADS / 32);  // 32-bit words of level bits per tile
};

// ------------------------------------------------------------ pre-pass
// Histogram of the top K of the L key bits, privatized in shared memory.

template <typename T>
__global__ void __launch_bounds__(256) prehist_kernel(const T* __restrict__ s, uint64_t n, int L, int K,
                                                      int vec_ok, uint32_t* __restrict__ hist) {
  extern __shared__ uint32_t sh[];
  const uint32_t bins = 1u << K;
  const uint64_t bmask = bins - 1;
  const int sh_r = L - K;
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  // whole warps step together so that equal bins of a warp are added once
  auto add = [&](bool valid, uint32_t key) {
    const uint32_t k = valid ? key : 0xFFFFFFFFu;
    const uint32_t grp = __match_any_sync(0xffffffffu, k);
    if (valid && lane == (uint32_t)(__ffs(grp) - 1)) atomicAdd(&sh[key], (uint32_t)__popc(grp));
  };
  const uint64_t wstride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t w0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
  constexpr int V = 16 / sizeof(T);
  uint64_t done = 0;
  if (vec_ok) {
    const uint64_t nv = n / V;
    const uint4* s4 = (const uint4*)s;
    for (uint64_t b = w0; b < nv; b += wstride) {
      const uint64_t i = b + lane;
      const bool valid = i < nv;
      uint4 q = valid ? __ldg(&s4[i]) : make_uint4(0, 0, 0, 0);
      const T* e = (const T*)&q;
#pragma unroll
      for (int k = 0; k < V; ++k) add(valid, (uint32_t)(((uint64_t)e[k] >> sh_r) & bmask));
    }
    done = nv * V;
  }
  for (uint64_t b = done + w0; b < n; b += wstride) {
    const uint64_t i = b + lane;
    const bool valid = i < n;
    add(valid, valid ? (uint32_t)(((uint64_t)s[i] >> sh_r) & bmask) : 0u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
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

__device__ __forceinline__ void emit_flush(uint32_t* __restrict__ znext, uint32_t p, uint32_t ce, uint32_t co) {
  if (p == 0xFFFFFFFFu) return;
  if (ce) atomicAdd(&znext[2 * p], ce);
  if (co) atomicAdd(&znext[2 * p + 1], co);
}

// One level: bits of level `level` for every symbol of the level order in
// src, and (SCATTER) the stable partition of src into dst, and (EMIT) the
// zero counts of the level+1 nodes.
template <typename T, bool SCATTER, bool EMIT>
__global__ void __launch_bounds__(LV_THREADS)
    level_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, int L, int level,
                 const uint2* __restrict__ base_lvl, uint32_t* __restrict__ bits32, uint64_t bit_off,
                 uint64_t* status, uint32_t* counter, uint32_t* err, uint32_t* __restrict__ znext, int bulk_ok) {
  using S = LvShape<T>;
  extern __shared__ __align__(128) unsigned char lv_smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_tile[2];
  __shared__ uint32_t s_cnt[S::NW];
  __shared__ uint32_t s_bits[S::NW];
  __shared__ uint32_t s_prefix;
  T* const buf0 = (T*)lv_smem;
  T* const buf1 = (T*)(lv_smem + S::BYTES);
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t ntiles = (n + S::TILE - 1) / S::TILE;
  const uint64_t nfull = bulk_ok ? n / S::TILE : 0;  // tiles fetched with bulk copies
  const int shift = L - 1 - level;
  const uint32_t pmask = level ? (uint32_t)((1ull << level) - 1) : 0u;

  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_fence_init();
    const uint32_t t0 = atomicAdd(counter, 1u);
    s_tile[0] = t0;
    if (t0 < nfull) {
      mbar_expect_tx(&mbar[0], S::BYTES);
      bulk_g2s(buf0, src + (uint64_t)t0 * S::TILE, S::BYTES, &mbar[0]);
    }
  }
  __syncthreads();
  uint32_t phase0 = 0, phase1 = 0;
  int cur = 0;
  for (;;) {
    const uint32_t tile = s_tile[cur];
    if (tile >= ntiles) break;
    if (tid == 0) {  // prefetch the next tile into the other buffer
      const uint32_t nt = atomicAdd(counter, 1u);
      s_tile[cur ^ 1] = nt;
      if (nt < nfull) {
        fence_proxy_async_smem();
        mbar_expect_tx(&mbar[cur ^ 1], S::BYTES);
        bulk_g2s(cur ? buf0 : buf1, src + (uint64_t)nt * S::TILE, S::BYTES, &mbar[cur ^ 1]);
      }
    }
    T* const tb = cur ? buf1 : buf0;
    const uint64_t tile_base = (uint64_t)tile * S::TILE;
    if (tile < nfull) {
      if (cur) {
        mbar_wait(&mbar[1], phase1, err);
        phase1 ^= 1;
      } else {
        mbar_wait(&mbar[0], phase0, err);
        phase0 ^= 1;
      }
    } else {
      for (uint32_t k = tid; k < S::TILE; k += LV_THREADS) {
        const uint64_t i = tile_base + k;
        tb[k] = i < n ? src[i] : T(0);
      }
      __syncthreads();
    }

    // 1. level bits and zero counts per (row, warp); next-level zero counts
    uint32_t run_p = 0xFFFFFFFFu, c_even = 0, c_odd = 0;
#pragma unroll 4
    for (int r = 0; r < S::ROWS; ++r) {
      const uint32_t k = r * LV_THREADS + tid;
      const bool valid = tile_base + k < n;
      const uint64_t x = valid ? (uint64_t)tb[k] : 0ull;
      const bool one = valid && ((x >> shift) & 1);
      const uint32_t ones = __ballot_sync(0xffffffffu, one);
      const uint32_t zeros = __ballot_sync(0xffffffffu, valid && !one);
      if (lane == 0) {
        s_bits[r * 8 + warp] = ones;
        s_cnt[r * 8 + warp] = __popc(zeros);
      }
      if (EMIT) {
        const uint32_t p = level ? ((uint32_t)(x >> (L - level)) & pmask) : 0u;
        const bool zn = valid && !((x >> (shift - 1)) & 1);
        const uint32_t p0 = __shfl_sync(0xffffffffu, p, 0);
        if (__ballot_sync(0xffffffffu, valid && p != p0) == 0) {
          const uint32_t ce = __popc(__ballot_sync(0xffffffffu, zn && !one));
          const uint32_t co = __popc(__ballot_sync(0xffffffffu, zn && one));
          if (p0 != run_p) {
            if (lane == 0) emit_flush(znext, run_p, c_even, c_odd);
            run_p = p0;
            c_even = c_odd = 0;
          }
          c_even += ce;
          c_odd += co;
        } else {
          const uint32_t key = zn ? (2 * p + (one ? 1u : 0u)) : 0xFFFFFFFFu;
          const uint32_t grp = __match_any_sync(0xffffffffu, key);
          if (zn && lane == (uint32_t)(__ffs(grp) - 1)) atomicAdd(&znext[key], (uint32_t)__popc(grp));
        }
      }
    }
    if (EMIT && lane == 0) emit_flush(znext, run_p, c_even, c_odd);
    __syncthreads();

    // 2. store the bits: tile word j covers global bits [g + 32 j, g + 32 j + 32)
    {
      const uint64_t g = bit_off + tile_base;
      const uint32_t g0 = (uint32_t)(g & 31);
      const uint64_t G = g >> 5;
      const uint64_t valid_bits = min((uint64_t)S::TILE, n - tile_base);
      for (int j = tid; j <= S::NW; j += LV_THREADS) {
        if (g0 == 0 && j == S::NW) break;
        const uint32_t curw = j < S::NW ? s_bits[j] : 0u;
        const uint32_t prev = j > 0 ? s_bits[j - 1] : 0u;
        const uint32_t val = g0 ? ((curw << g0) | (prev >> (32 - g0))) : curw;
        const uint64_t wlo = (G + j) * 32;
        if (wlo >= g + valid_bits) continue;
        const bool full = (wlo >= g) && (wlo + 32 <= g + valid_bits);
        if (full) bits32[G + j] = val;
        else if (val) atomicOr(&bits32[G + j], val);
      }
    }

    if (SCATTER) {
      // 3. tile-exclusive zero counts and the tile's prefix (look-back)
      if (warp == 0) {
        constexpr int PER = S::NW / 32;
        uint32_t loc[PER];
        uint32_t sum = 0;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          loc[q] = s_cnt[lane * PER + q];
          sum += loc[q];
        }
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= (uint32_t)o) inc += t;
        }
        uint32_t run = inc - sum;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          s_cnt[lane * PER + q] = run;
          run += loc[q];
        }
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        uint64_t prefix = 0;
        if (tile == 0) {
          if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, total);
        } else {
          if (lane == 0) lb_publish(status, tile, LB_FLAG_AGG, total);
          prefix = lb_lookback_warp(status, tile, err);
          if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, prefix + total);
        }
        if (lane == 0) s_prefix = (uint32_t)prefix;
      }
      __syncthreads();

      // 4. stable partition: scatter into the next level's order
      const uint32_t zprefix = s_prefix;
      const uint32_t ltmask = lanemask_lt();
#pragma unroll 4
      for (int r = 0; r < S::ROWS; ++r) {
        const uint32_t k = r * LV_THREADS + tid;
        const uint64_t i = tile_base + k;
        const bool valid = i < n;
        const T x = tb[k];
        const bool one = valid && (((uint64_t)x >> shift) & 1);
        const uint32_t zm = __ballot_sync(0xffffffffu, valid && !one);
        if (valid) {
          const uint32_t z_before = zprefix + s_cnt[r * 8 + warp] + __popc(zm & ltmask);
          const uint32_t p = level ? ((uint32_t)((uint64_t)x >> (L - level)) & pmask) : 0u;
          const uint2 b = base_lvl[p];
          const uint32_t d = one ? b.y + ((uint32_t)i - z_before) : b.x + z_before;
          if (d < n) dst[d] = x;
          else atomicCAS(err, 0u, (uint32_t)DERR_BAD_INDEX);
        }
      }
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
static void launch_prehist(const void* s, uint64_t n, int L, int K, uint32_t* hist, cudaStream_t st) {
  unsigned grid = (unsigned)std::min<uint64_t>((n / (16 / sizeof(T)) + 255) / 256, (uint64_t)sm_count() * 4);
  if (grid == 0) grid = 1;
  const int vec_ok = ((uintptr_t)s % 16) == 0;
  prehist_kernel<T><<<grid, 256, sizeof(uint32_t) << K, st>>>((const T*)s, n, L, K, vec_ok, hist);
}

template <typename T>
static void launch_max(const void* s, uint64_t n, unsigned long long* out, cudaStream_t st) {
  unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8);
  if (grid == 0) grid = 1;
  max_kernel<T><<<grid, 256, 0, st>>>((const T*)s, n, out);
}

template <typename T, bool SC, bool EM>
static int level_grid(uint64_t n) {
  static int per_sm = 0;
  if (!per_sm) {
    cudaFuncSetAttribute(level_kernel<T, SC, EM>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, level_kernel<T, SC, EM>, LV_THREADS,
                                                  2 * LvShape<T>::BYTES);
    if (per_sm <= 0) per_sm = 1;
  }
  const uint64_t tiles = (n + LvShape<T>::TILE - 1) / LvShape<T>::TILE;
  return (int)std::min<uint64_t>(tiles, (uint64_t)per_sm * sm_count());
}

template <typename T>
static void launch_level(const void* src, void* dst, uint64_t n, int L, int level, const uint2* base_lvl,
                         uint32_t* bits32, uint64_t bit_off, uint64_t* status, uint32_t* counter, uint32_t* err,
                         uint32_t* znext, bool scatter, bool emit, cudaStream_t st) {
  const int bulk_ok = ((uintptr_t)src % 16) == 0;
  const size_t shm = 2 * LvShape<T>::BYTES;
#define WTG_LV(SC, EM)                                                                                       \
  level_kernel<T, SC, EM><<<level_grid<T, SC, EM>(n), LV_THREADS, shm, st>>>(                               \
      (const T*)src, (T*)dst, n, L, level, base_lvl, bits32, bit_off, status, counter, err, znext, bulk_ok)
  if (scatter && emit) WTG_LV(true, true);
  else if (scatter) WTG_LV(true, false);
  else WTG_LV(false, false);
#undef WTG_LV
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
  if (n) {
    prof_begin(PROF_HIST, s);
    WTG_DISPATCH(eb, launch_prehist, d_seq, n, L, K, S, s);
    prof_end(PROF_HIST, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  if ((rc = scan_exclusive_u32(S, S, (1ull << K) + 1, t.scan_tmp, d_err, s))) return rc;
  {
    const uint64_t top = (1ull << K) - 1;
    unsigned grid = (unsigned)std::min<uint64_t>((top + 255) / 256, 1024);
    if (grid == 0) grid = 1;
    prof_begin(PROF_TABLES, s);
    top_tables_kernel<<<grid, 256, 0, s>>>(S, K, C, Z);
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = scan_exclusive_u32(Z, ZS, top + 1, t.scan_tmp, d_err, s))) return rc;
    prof_begin(PROF_TABLES, s);
    base_kernel<<<grid, 256, 0, s>>>(C, Z, ZS, K, base);
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }

  // level passes; levels >= K get their tables from the previous pass
  if (n) {
    const uint64_t tiles = (n + tile_elems(eb) - 1) / tile_elems(eb);
    const uint64_t per_level = tiles + 1;
    if ((rc = t.status.ensure(per_level * (uint64_t)L * sizeof(uint64_t), s))) return rc;
    WTG_CK(cudaMemsetAsync(t.status.p, 0, per_level * (uint64_t)L * sizeof(uint64_t), s));
    if (L > 1) {
      if ((rc = t.lvl[0].ensure(n * eb + 16, s))) return rc;
      if ((rc = t.lvl[1].ensure(n * eb + 16, s))) return rc;
    }
    const void* src = d_seq;
    for (int l = 0; l < L; ++l) {
      const bool scatter = l < L - 1;
      const bool emit = (l + 1 >= K) && (l + 1 <= L - 2);
      void* dst = scatter ? t.lvl[l & 1].p : nullptr;
      uint64_t* st = t.status.as<uint64_t>() + per_level * l;
      uint32_t* znext = Z + ((1ull << (l + 1)) - 1);
      prof_begin(scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      WTG_DISPATCH(eb, launch_level, src, dst, n, L, l, base + ((1ull << l) - 1), t.bits.as<uint32_t>(),
                   (uint64_t)l * n, st + 1, (uint32_t*)st, d_err, znext, scatter, emit, s);
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
