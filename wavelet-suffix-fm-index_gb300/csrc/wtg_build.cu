// wtg_build.cu -- level-by-level wavelet-tree construction on the GPU.
//
// The reference (wavelet/levelWT/WT.C:86-270) walks the tree node by node:
// at level l every node writes bit (levels-l-1) of its symbols at
// l*n + position and stably partitions them, zeros first, into the next
// level's buffer.  Here a level is one flat pass over the whole sequence:
//
//   * the level-l order is the input stably sorted by the top l bits of each
//     symbol, so node p of level l is the range [C_l(p), C_l(p+1)) of it, and
//     C_l comes from one histogram of the full keys (hist_kernel, scanned);
//   * the level's bits are a coalesced map: one __ballot_sync per warp and row
//     yields 32 bits, staged in shared memory and stored as whole words;
//   * the stable partition is a scatter: with Z(i) = number of zeros before
//     position i at this level (one decoupled look-back scan per level) an
//     element with bit 0 goes to  C_l(p) + Z(i) - Zb(p)  and one with bit 1 to
//     C_l(p) + zeros(p) + (i - Z(i)) - (C_l(p) - Zb(p)), where zeros(p) and
//     Zb(p) (zeros in nodes before p) come from the same histogram;
//     base_kernel folds them into two per-node constants.
//
// Each level therefore reads and writes the sequence once and writes n/8
// bytes of bits; the node table (WT.C:110,156-159,234-257) follows from the
// histogram alone.
#include <algorithm>

#include "wtg_internal.cuh"
#include "wtg_tree.cuh"

namespace wtg {

constexpr int LV_THREADS = 256;
constexpr int LV_IPT = 16;
constexpr uint32_t LV_TILE = LV_THREADS * LV_IPT;

// ------------------------------------------------------------- histogram

template <typename T>
__global__ void __launch_bounds__(256) hist_kernel(const T* __restrict__ s, uint64_t n, int L,
                                                   uint32_t* __restrict__ hist) {
  extern __shared__ uint32_t sh[];
  const uint64_t mask = (1ull << L) - 1;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (L <= 12) {
    const uint32_t bins = 1u << L;
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
      atomicAdd(&sh[(uint64_t)s[i] & mask], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
  } else {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
      atomicAdd(&hist[(uint64_t)s[i] & mask], 1u);
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
// S = exclusive scan of the key histogram (S[2^L] = n).

__device__ __forceinline__ void heap_split(uint64_t h, int& l, uint64_t& p) {
  l = 63 - __clzll((long long)(h + 1));
  p = h + 1 - (1ull << l);
}

// zeros(h): symbols of node h whose level bit is 0 (its left child's size)
__global__ void zeros_kernel(const uint32_t* __restrict__ S, int L, uint32_t* __restrict__ Z) {
  const uint64_t total = 1ull << L;
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < total;
       h += (uint64_t)gridDim.x * blockDim.x) {
    if (h + 1 == total) {
      Z[h] = 0;
      continue;
    }
    int l;
    uint64_t p;
    heap_split(h, l, p);
    Z[h] = S[(2 * p + 1) << (L - l - 1)] - S[p << (L - l)];
  }
}

// base(h) = (C - Zb, zeros + Zb), Zb = zeros of the level's nodes before h
__global__ void base_kernel(const uint32_t* __restrict__ S, const uint32_t* __restrict__ Z,
                            const uint32_t* __restrict__ ZS, int L, uint2* __restrict__ base) {
  const uint64_t total = (1ull << L) - 1;
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < total;
       h += (uint64_t)gridDim.x * blockDim.x) {
    int l;
    uint64_t p;
    heap_split(h, l, p);
    uint32_t zb = ZS[h] - ZS[(1ull << l) - 1];
    uint32_t c = S[p << (L - l)];
    base[h] = make_uint2(c - zb, Z[h] + zb);
  }
}

// WTnode records in heap order (levelWT/WT.C:89-110,156-159,234-257).
__global__ void node_kernel(const uint32_t* __restrict__ S, const uint32_t* __restrict__ Z, int L, uint64_t n,
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
    uint32_t start = S[p << (L - l)];
    uint32_t len = S[(p + 1) << (L - l)] - start;
    if (h == 0 || len > 0) {
      rec[0] = (uint64_t)l * n + start;
      rec[1] = len;
      rec[2] = h == 0 ? none : (h - 1) / 2;
      if (l < L - 1) {
        uint32_t z = Z[h];
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

template <typename T, bool SCATTER>
__global__ void __launch_bounds__(LV_THREADS)
    level_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, int L, int level,
                 const uint2* __restrict__ base_lvl, uint32_t* __restrict__ bits32, uint64_t bit_off,
                 uint64_t* status, uint32_t* counter, uint32_t* err) {
  constexpr int NW = LV_IPT * (LV_THREADS / 32);  // 32-bit words of bits per tile
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_cnt[NW];
  __shared__ uint32_t s_bits[NW];
  __shared__ uint32_t s_prefix;

  if (threadIdx.x == 0) s_tile = SCATTER ? atomicAdd(counter, 1u) : blockIdx.x;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t tile_base = (uint64_t)tile * LV_TILE;
  const int shift = L - 1 - level;

  T v[LV_IPT];
  uint32_t zm[LV_IPT];
#pragma unroll
  for (int r = 0; r < LV_IPT; ++r) {
    const uint64_t i = tile_base + (uint64_t)r * LV_THREADS + threadIdx.x;
    const bool valid = i < n;
    const T x = valid ? src[i] : T(0);
    v[r] = x;
    const bool one = valid && (((uint64_t)x >> shift) & 1);
    const uint32_t ones = __ballot_sync(0xffffffffu, one);
    const uint32_t zeros = __ballot_sync(0xffffffffu, valid && !one);
    zm[r] = zeros;
    if (lane == 0) {
      s_bits[r * 8 + warp] = ones;
      s_cnt[r * 8 + warp] = __popc(zeros);
    }
  }
  __syncthreads();

  // bits: tile word j covers global bits [g + 32 j, g + 32 j + 32)
  {
    const uint64_t g = bit_off + tile_base;
    const uint32_t g0 = (uint32_t)(g & 31);
    const uint64_t G = g >> 5;
    const uint64_t valid_bits = min((uint64_t)LV_TILE, n - tile_base);
    for (int j = threadIdx.x; j <= NW; j += LV_THREADS) {
      if (g0 == 0 && j == NW) break;
      const uint32_t cur = j < NW ? s_bits[j] : 0u;
      const uint32_t prev = j > 0 ? s_bits[j - 1] : 0u;
      const uint32_t val = g0 ? ((cur << g0) | (prev >> (32 - g0))) : cur;
      const uint64_t wlo = (G + j) * 32;
      if (wlo >= g + valid_bits) continue;
      const bool full = (wlo >= g) && (wlo + 32 <= g + valid_bits);
      if (full) bits32[G + j] = val;
      else if (val) atomicOr(&bits32[G + j], val);
    }
  }

  if (!SCATTER) return;

  if (warp == 0) {
    constexpr int PER = NW / 32;
    uint32_t loc[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      loc[k] = s_cnt[lane * PER + k];
      sum += loc[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (uint32_t)o) inc += t;
    }
    uint32_t run = inc - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      s_cnt[lane * PER + k] = run;
      run += loc[k];
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

  const uint32_t zprefix = s_prefix;
  const uint32_t ltmask = lanemask_lt();
  const uint32_t pmask = level ? ((1u << level) - 1) : 0u;
#pragma unroll
  for (int r = 0; r < LV_IPT; ++r) {
    const uint64_t i = tile_base + (uint64_t)r * LV_THREADS + threadIdx.x;
    if (i < n) {
      const T x = v[r];
      const bool one = ((uint64_t)x >> shift) & 1;
      const uint32_t z_before = zprefix + s_cnt[r * 8 + warp] + __popc(zm[r] & ltmask);
      const uint32_t p = level ? ((uint32_t)((uint64_t)x >> (L - level)) & pmask) : 0u;
      const uint2 b = base_lvl[p];
      const uint32_t d = one ? b.y + ((uint32_t)i - z_before) : b.x + z_before;
      if (d < n) dst[d] = x;
      else atomicCAS(err, 0u, (uint32_t)DERR_BAD_INDEX);
    }
  }
}

// ------------------------------------------------------------------ host

template <typename T>
static void launch_hist(const void* s, uint64_t n, int L, uint32_t* hist, cudaStream_t st) {
  unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 8);
  if (grid == 0) grid = 1;
  size_t shm = L <= 12 ? (sizeof(uint32_t) << L) : 0;
  hist_kernel<T><<<grid, 256, shm, st>>>((const T*)s, n, L, hist);
}

template <typename T>
static void launch_max(const void* s, uint64_t n, unsigned long long* out, cudaStream_t st) {
  unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 8);
  if (grid == 0) grid = 1;
  max_kernel<T><<<grid, 256, 0, st>>>((const T*)s, n, out);
}

template <typename T>
static void launch_level(const void* src, void* dst, uint64_t n, int L, int level, const uint2* base_lvl,
                         uint32_t* bits32, uint64_t bit_off, uint64_t* status, uint32_t* counter, uint32_t* err,
                         bool scatter, cudaStream_t st) {
  unsigned tiles = (unsigned)((n + LV_TILE - 1) / LV_TILE);
  if (scatter)
    level_kernel<T, true><<<tiles, LV_THREADS, 0, st>>>((const T*)src, (T*)dst, n, L, level, base_lvl, bits32,
                                                        bit_off, status, counter, err);
  else
    level_kernel<T, false><<<tiles, LV_THREADS, 0, st>>>((const T*)src, (T*)dst, n, L, level, base_lvl, bits32,
                                                         bit_off, status, counter, err);
}

#define WTG_DISPATCH(eb, fn, ...)                       \
  switch (eb) {                                         \
    case 1: fn<uint8_t>(__VA_ARGS__); break;            \
    case 2: fn<uint16_t>(__VA_ARGS__); break;           \
    case 4: fn<uint32_t>(__VA_ARGS__); break;           \
    default: fn<uint64_t>(__VA_ARGS__); break;          \
  }

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
  const uint64_t bins = 1ull << L;

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

  // key histogram -> S (exclusive scan, S[2^L] = n)
  if ((rc = t.hist.ensure((bins + 1) * sizeof(uint32_t), s))) return rc;
  if ((rc = t.zeros.ensure(2 * bins * sizeof(uint32_t), s))) return rc;  // [Z | ZS]
  if ((rc = t.base.ensure(bins * sizeof(uint2), s))) return rc;
  uint32_t* S = t.hist.as<uint32_t>();
  uint32_t* Z = t.zeros.as<uint32_t>();
  uint32_t* ZS = Z + bins;
  WTG_CK(cudaMemsetAsync(S, 0, (bins + 1) * sizeof(uint32_t), s));
  if (n) {
    prof_begin(PROF_HIST, s);
    WTG_DISPATCH(eb, launch_hist, d_seq, n, L, S, s);
    prof_end(PROF_HIST, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  if ((rc = scan_exclusive_u32(S, S, bins + 1, t.scan_tmp, d_err, s))) return rc;
  {
    unsigned grid = (unsigned)std::min<uint64_t>((bins + 255) / 256, 152 * 16);
    prof_begin(PROF_TABLES, s);
    zeros_kernel<<<grid, 256, 0, s>>>(S, L, Z);
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = scan_exclusive_u32(Z, ZS, bins, t.scan_tmp, d_err, s))) return rc;
    prof_begin(PROF_TABLES, s);
    base_kernel<<<grid, 256, 0, s>>>(S, Z, ZS, L, t.base.as<uint2>());
    prof_end(PROF_TABLES, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }

  // level passes
  if (n) {
    const uint64_t tiles = (n + LV_TILE - 1) / LV_TILE;
    const uint64_t per_level = tiles + 1;
    if ((rc = t.status.ensure(per_level * (uint64_t)L * sizeof(uint64_t), s))) return rc;
    WTG_CK(cudaMemsetAsync(t.status.p, 0, per_level * (uint64_t)L * sizeof(uint64_t), s));
    if (L > 1) {
      if ((rc = t.lvl[0].ensure(n * eb, s))) return rc;
      if ((rc = t.lvl[1].ensure(n * eb, s))) return rc;
    }
    const void* src = d_seq;
    for (int l = 0; l < L; ++l) {
      const bool scatter = l < L - 1;
      void* dst = scatter ? t.lvl[l & 1].p : nullptr;
      uint64_t* st = t.status.as<uint64_t>() + per_level * l;
      prof_begin(scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      WTG_DISPATCH(eb, launch_level, src, dst, n, L, l, t.base.as<uint2>() + ((1ull << l) - 1),
                   t.bits.as<uint32_t>(), (uint64_t)l * n, st + 1, (uint32_t*)st, d_err, scatter, s);
      prof_end(scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      count_launch();
      WTG_CK(cudaGetLastError());
      src = dst;
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
  unsigned grid = (unsigned)((n_entries + 255) / 256);
  node_kernel<<<grid, 256, 0, s>>>(t.hist.as<uint32_t>(), t.zeros.as<uint32_t>(), t.levels, t.n, n_entries, ib,
                                   d_out);
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
