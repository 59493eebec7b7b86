// wtg_build.cu -- level-by-level wavelet-tree construction on the GPU.
//
// The reference (wavelet/levelWT/WT.C:43-227) walks the tree node by node:
// at level l every node writes bit (levels-l-1) of its symbols at
// l*n + position and stably partitions them, zeros first, into the next
// level's buffer.  Here a level is one flat pass over the whole sequence:
//
//   * the level-l order is the input stably sorted by the top l bits of each
//     symbol, so node p of level l is the range [C_l(p), C_l(p+1)) of it;
//   * the level's bits are a coalesced map: one __ballot_sync per warp and row
//     yields 32 bits, staged in shared memory and stored as whole words;
//   * the stable partition is a scatter: with Z(i) = number of zeros before
//     position i at this level, an element of node p with bit 0 goes to
//     C_l(p) + Z(i) - Zb(p)  and one with bit 1 to
//     C_l(p) + zeros(p) + (i - Z(i)) - (C_l(p) - Zb(p)), where zeros(p) is
//     the size of p's left child and Zb(p) the zeros of the level's nodes
//     before p; base_kernel / level_table_kernel fold them into two per-node
//     constants.  Z at every 512-symbol chunk start is the exclusive scan of
//     the per-chunk zero counts the previous pass emitted for its
//     destination chunks (level 0: the pre-pass), so no pass waits on
//     another chunk's result.
//
// Node sizes: the pre-pass histograms the top K = 2 bits, which gives C and
// zeros for levels 0 and 1.  For deeper levels the pass over level l counts,
// per node of level l+1, the symbols whose next bit is 0: a chunk inside one
// node p stores its two counts (nodes 2p, 2p+1) per chunk, a scan and
// node_sum_kernel add them up per node, and chunks across node boundaries
// add theirs with atomics; level_table_kernel then derives level l+1's
// constants before its pass.
//
// Each level pass is a persistent kernel in which every warp runs its own
// pipeline: it fetches groups of 512-symbol chunks (4 KB) with cp.async.bulk
// into a private two-stage ring and waits on its own mbarriers, the chunks of
// the level taken in a grid stride (a narrow moving window of the order, so
// the writes advance in a few dense fronts).  Per level the sequence is read
// once and written once, plus n/8 bytes of bits.  The node table
// (WT.C:67,113-116,191-214) follows from the per-node starts and zero counts
// alone.
#include <algorithm>
#include <type_traits>

#include "wtg_internal.cuh"
#include "wtg_tree.cuh"

namespace wtg {

WTG_WAIT_LIMIT_SETTER(build)

constexpr int LV_THREADS = 256;
// chunk-group buffers per warp (prefetch depth + 1)
template <bool SCATTER>
constexpr int lv_stages() { return 2; }
constexpr int TOP_BITS = 2;  // bits histogrammed by the pre-pass (ballot counted)

constexpr int CHUNK = 512;      // symbols per warp chunk (16 rows of 32)
constexpr int LOG_CHUNK = 9;
constexpr int WROWS = CHUNK / 32;

// A warp fetches CPB consecutive chunks with one 4 KB cp.async.bulk: on
// GB300 a ring of 2 KB bulk copies reads at about 3.5 TB/s, one of 4 KB
// copies at 6.8-7.4 TB/s (the per-copy cost, not the bytes, sets the rate).
template <typename T>
struct LvShape {
  static constexpr uint32_t CPB = CHUNK * sizeof(T) >= 4096 ? 1 : 4096 / (CHUNK * sizeof(T));
  static constexpr uint32_t TILE = LV_THREADS / 32 * CHUNK;  // symbols per CTA tile
  static constexpr uint32_t BYTES = TILE * sizeof(T) * CPB;  // one chunk group per warp
  template <bool SCATTER>
  static constexpr uint32_t smem() { return lv_stages<SCATTER>() * BYTES; }  // the warps' rings
};

// ------------------------------------------------------------ pre-pass
// One read of the input: the zero count of level 0 (bit levels-1) in every
// 512-symbol chunk, and the histogram of the top K <= 2 key bits.  A warp per
// chunk, 16-byte coalesced loads of two chunks in flight per warp, counts
// kept in registers.

template <typename T>
__global__ void __launch_bounds__(LV_THREADS) prepass_kernel(const T* __restrict__ s, uint64_t n, int L, int K,
                                                             int vec_ok, uint64_t c_begin, uint64_t c_end,
                                                             uint32_t* __restrict__ chunkcnt,
                                                             uint32_t* __restrict__ hist) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const int top = L - 1;
  const int top2 = K > 1 ? L - 2 : 0;
  uint32_t c1 = 0, c2 = 0, c12 = 0, cnt = 0;  // top bit set, second bit set, both, symbols
  constexpr int PER = 16 / sizeof(T);
  constexpr int NV = CHUNK * sizeof(T) / 16 / 32;  // 16-byte loads per lane and chunk
  auto take = [&](uint64_t x, uint32_t& ones) {
    const uint32_t b1 = (uint32_t)(x >> top) & 1u;
    const uint32_t b2 = K > 1 ? (uint32_t)(x >> top2) & 1u : 0u;
    ones += b1;
    c2 += b2;
    c12 += b1 & b2;
  };
  // one chunk's counts from its preloaded vectors (full) or scalar loads
  auto chunk = [&](uint64_t c, bool full, const uint4* v) {
    const uint64_t base = c * CHUNK;
    const uint32_t cv = (uint32_t)min((uint64_t)CHUNK, n - base);
    uint32_t ones = 0;
    if (full) {
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const T* e = (const T*)&v[j];
#pragma unroll
        for (int k = 0; k < PER; ++k) take((uint64_t)e[k], ones);
      }
      cnt += CHUNK / 32;
    } else {
      for (uint32_t k = lane; k < cv; k += 32) {
        take((uint64_t)s[base + k], ones);
        ++cnt;
      }
    }
    c1 += ones;
    const uint32_t wz = __reduce_add_sync(0xffffffffu, ones);
    if (lane == 0) chunkcnt[c] = cv - wz;  // zeros of level 0 in this chunk
  };
  // chunks c_begin..c_end-1, two per step, both loaded before either is counted
  for (uint64_t c = c_begin + gw; c < c_end; c += 2 * nwarps) {
    const uint64_t cb = c + nwarps;
    const bool fa = vec_ok && (c + 1) * CHUNK <= n;
    const bool fb = vec_ok && cb < c_end && (cb + 1) * CHUNK <= n;
    uint4 va[NV], vb[NV];
    if (fa) {
      const uint4* q = (const uint4*)(s + c * CHUNK);
#pragma unroll
      for (int j = 0; j < NV; ++j) va[j] = __ldg(&q[j * 32 + lane]);
    }
    if (fb) {
      const uint4* q = (const uint4*)(s + cb * CHUNK);
#pragma unroll
      for (int j = 0; j < NV; ++j) vb[j] = __ldg(&q[j * 32 + lane]);
    }
    chunk(c, fa, va);
    if (cb < c_end) chunk(cb, fb, vb);
  }
  // bins of the top K bits (K = 1: bins 0/1 = top bit 0/1)
  uint32_t h[4] = {cnt - c1 - c2 + c12, c2 - c12, c1 - c12, c12};
#pragma unroll
  for (int b2 = 0; b2 < 4; ++b2)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h[b2] += __shfl_xor_sync(0xffffffffu, h[b2], o);
  if (lane == 0) {
    if (K > 1) {
      for (int b2 = 0; b2 < 4; ++b2)
        if (h[b2]) atomicAdd(&hist[b2], h[b2]);
    } else {
      if (h[0]) atomicAdd(&hist[0], h[0]);
      if (h[2]) atomicAdd(&hist[1], h[2]);
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
// Heap id h = 2^l - 1 + p names node p of level l (levelWT/WT.C:191-214).
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

// WTnode records in heap order (levelWT/WT.C:46-67,113-116,191-214).
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

// node of a symbol: 32-bit shifts for symbols of up to 4 bytes, 64-bit otherwise
template <typename T>
__device__ __forceinline__ uint32_t prefix_of(T x, int s, uint32_t mask) {
  if constexpr (sizeof(T) <= 4) return (s >= 32 ? 0u : ((uint32_t)x >> s)) & mask;
  else return (uint32_t)((uint64_t)x >> s) & mask;
}

// One level over the level-l order in src.  Every warp runs its own
// pipeline over groups of CPB consecutive 512-symbol chunks (4 KB; group =
// global warp id + k * warps): it prefetches its next group with one
// cp.async.bulk into the other half of its private double buffer and waits
// on its own mbarrier, so warps never synchronise with each other.  A
// chunk's zeros-before come from chunkpre (the scan of the counts the
// previous pass emitted), read for the whole group before the wait.  Per
// chunk:
//   * the level's bits: one ballot per 32 symbols, stored as whole words;
//   * SCATTER: every symbol goes straight to its place in the next level's
//     order: bit 0 -> C(p) + zeros before it in node p, bit 1 ->
//     C(p) + zeros(p) + ones before it in node p, through base(p) =
//     (C - Zb, zeros + Zb) and the level-wide zero rank;
//   * EMIT_TILES: per 512-symbol chunk of the next level, the number of its
//     symbols whose next bit is 0 (the next pass's chunkpre input);
//   * EMIT_NODES: per node of the next level, its left-child size: a chunk
//     inside one node p stores its two counts (for nodes 2p and 2p+1) in
//     nc0[c], nc1[c], which the host-side scans and node_sum_kernel add up
//     per node; a chunk across node boundaries adds its counts with atomics.
//     (Counting with per-warp runs and atomics on the node counters put
//     one atomic per group on the few nodes a grid stride spans at the
//     middle levels -- a hot L2 slice that slowed those levels by a third.)
// A full chunk inside one node (the common case) takes a lean unrolled path:
// one base(p), its zero run and one run contiguous in dst, each touching at
// most two destination chunks, so emission is per-row counting, one ballot
// for the row that holds a destination boundary, and four atomics per chunk.
// Other chunks take a compact general path.
template <typename T, bool SCATTER, bool EMIT_NODES, bool EMIT_TILES>
__global__ void __launch_bounds__(LV_THREADS, 3)
    level_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, int L, int level,
                 const uint2* __restrict__ base_lvl, uint32_t* __restrict__ bits32, uint64_t bit_off,
                 const uint32_t* __restrict__ chunkpre, uint32_t* __restrict__ chunkcnt_next,
                 uint32_t* __restrict__ nc0, uint32_t* __restrict__ nc1,
                 uint32_t* __restrict__ znext, uint32_t* err, int bulk_ok, uint32_t* __restrict__ chunkcnt_self) {
  constexpr uint32_t CBYTES = CHUNK * sizeof(T);
  constexpr uint32_t CPB = LvShape<T>::CPB;
  constexpr uint32_t GBYTES = CBYTES * CPB;  // one bulk copy: CPB consecutive chunks
  constexpr int LV_STAGES = lv_stages<SCATTER>();
  extern __shared__ __align__(128) unsigned char lv_smem[];
  __shared__ __align__(8) uint64_t mbar[LV_THREADS / 32][LV_STAGES];
  __shared__ uint2 s_rows[LV_THREADS / 32][WROWS];  // per row: its bits, its next-level zero mask
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* const wring = (T*)(lv_smem + warp * LV_STAGES * GBYTES);  // this warp's LV_STAGES group buffers
  uint64_t* const bars = mbar[warp];
  uint2* const myrow = s_rows[warp];
  const uint64_t nchunks = (n + CHUNK - 1) / CHUNK;
  const uint64_t ngroups = (nchunks + CPB - 1) / CPB;
  const uint64_t nfullg = bulk_ok ? n / (CHUNK * CPB) : 0;  // groups fetched with bulk copies
  const uint64_t stride = (uint64_t)gridDim.x * (LV_THREADS / 32);
  const uint64_t g0 = (uint64_t)blockIdx.x * (LV_THREADS / 32) + warp;
  const int shift = L - 1 - level;
  // L <= 24: the bits a pass tests lie in the low 32 bits of every symbol
  const uint32_t m1 = 1u << shift, mnext = m1 >> 1;
  const int pshift = L - level;
  const uint32_t pmask = level ? (uint32_t)((1ull << level) - 1) : 0u;
  const uint32_t ltmask = lanemask_lt();
  const uint32_t n32 = (uint32_t)n;  // n < 2^32

  // ring of LV_STAGES buffers: group number j (0, 1, ... of this warp) uses
  // slot j % LV_STAGES; LV_STAGES - 1 groups are in flight ahead of the one
  // being processed
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < LV_STAGES; ++q) mbar_init(&bars[q], 1);
    mbar_fence_init();
#pragma unroll
    for (int q = 0; q < LV_STAGES - 1; ++q) {
      const uint64_t gq = g0 + (uint64_t)q * stride;
      if (gq < nfullg) {
        mbar_expect_tx(&bars[q], GBYTES);
        bulk_g2s(wring + q * CPB * CHUNK, src + gq * CPB * CHUNK, GBYTES, &bars[q]);
      }
    }
  }
  __syncwarp();
  uint32_t phases = 0;  // bit q: parity of slot q's next completion
  int slot = 0;
  uint32_t cache_p = 0xFFFFFFFFu;  // base(p) cache
  uint2 cache_b = make_uint2(0, 0);
  for (uint64_t g = g0; g < ngroups; g += stride) {
    const uint64_t nx = g + (uint64_t)(LV_STAGES - 1) * stride;
    const int nslot = slot == 0 ? LV_STAGES - 1 : slot - 1;  // (slot + STAGES - 1) % STAGES
    if (lane == 0 && nx < nfullg) {  // refill the slot freed by the previous group
      fence_proxy_async_smem();
      mbar_expect_tx(&bars[nslot], GBYTES);
      bulk_g2s(wring + nslot * CPB * CHUNK, src + nx * CPB * CHUNK, GBYTES, &bars[nslot]);
    }
    // the group's chunk prefixes, loaded before the wait: lane j holds chunk g * CPB + j's
    uint32_t zpre_g = 0;
    if (SCATTER && lane < CPB && g * CPB + lane < nchunks) zpre_g = chunkpre[g * CPB + lane];
    const bool gbulk = g < nfullg;
    if (gbulk) {
      mbar_wait(&bars[slot], (phases >> slot) & 1u, err);
      phases ^= 1u << slot;
    }
#pragma unroll 1
  for (uint32_t j = 0; j < CPB; ++j) {
    const uint64_t c = g * CPB + j;
    if (c >= nchunks) break;
    T* const wt = wring + (slot * CPB + j) * CHUNK;
    const uint64_t cbase = c * CHUNK;
    const uint32_t cvalid = (uint32_t)min((uint64_t)CHUNK, n - cbase);
    if (!gbulk) {
      for (uint32_t k = lane; k < CHUNK; k += 32) wt[k] = k < cvalid ? src[cbase + k] : T(0);
      __syncwarp();
    }

    const uint32_t i0 = (uint32_t)cbase;
    bool bad = false;                          // a destination outside dst (inconsistent tables)
    uint32_t z = SCATTER ? __shfl_sync(0xffffffffu, zpre_g, j) : 0u;  // level-wide zeros before the chunk
    uint32_t p0 = 0;
    bool uniform = true;
    if (SCATTER && level) {
      p0 = prefix_of(wt[0], pshift, pmask);
      uniform = p0 == prefix_of(wt[cvalid - 1], pshift, pmask);  // the level order is sorted by node
    }

    if (!SCATTER) {
      // last level: bits only (and, when asked, the chunk's zero count)
      uint32_t zc = 0;
#pragma unroll 4
      for (int r = 0; r < WROWS; ++r) {
        const uint32_t k = r * 32 + lane;
        const bool valid = k < cvalid;
        const uint32_t om = __ballot_sync(0xffffffffu, valid && ((uint32_t)wt[k] & m1));
        myrow[r].x = om;  // every lane stores the same word: no branch
        zc += __popc(__ballot_sync(0xffffffffu, valid) & ~om);
      }
      if (chunkcnt_self && lane == 0) chunkcnt_self[c] = zc;
    } else if (uniform && cvalid == CHUNK) {
      // ---- fast path: full chunk inside one node
      if (p0 != cache_p) {
        cache_p = p0;
        cache_b = base_lvl[p0];
      }
      const uint2 b = cache_b;
      const uint32_t ob0 = i0 - z;                      // ones before the chunk
      const uint32_t zs = z;                            // zeros before the chunk
      // The chunk's zeros land in b.x + [zs, zs + 512) and its ones in
      // b.y + [ob0, ob0 + 512): when both ranges lie inside dst, no store of
      // the chunk needs its own check.
      const bool in_range = (uint64_t)b.x + zs + CHUNK <= n && (uint64_t)b.y + ob0 + CHUNK <= n;
      const uint32_t ybase = b.y + i0 + lane;  // a one at row r goes to ybase + 32 r - (zeros before it)
      auto rows = [&](auto checked) {
        constexpr bool CHECK = decltype(checked)::value;
#pragma unroll
        for (int r = 0; r < WROWS; ++r) {
          const T x = wt[r * 32 + lane];
          const bool one = (uint32_t)x & m1;
          const uint32_t om = __ballot_sync(0xffffffffu, one);
          const uint32_t zb = z + __popc(~om & ltmask);  // zeros before x (level-wide)
          z += 32u - __popc(om);
          const uint32_t d = one ? ybase + 32u * r - zb : b.x + zb;
          if (CHECK) {
            const bool okd = d < n32;
            if (okd) dst[d] = x;  // predicated; a bad index is reported after the chunk
            bad |= !okd;
          } else {
            dst[d] = x;
          }
          // every lane stores the same words: no branch
          if (EMIT_TILES) myrow[r] = make_uint2(om, __ballot_sync(0xffffffffu, !((uint32_t)x & mnext)));
          else myrow[r].x = om;
        }
      };
      if (in_range) rows(std::false_type{});
      else rows(std::true_type{});
      if (EMIT_TILES) {
        // Per 512-symbol chunk of the next level, its symbols whose next bit
        // is 0: the chunk's zero run lands at b.x + [zs, ...) and its one run
        // at b.y + [ob0, ...), each crossing at most one destination chunk
        // boundary (zero rank zlim, one rank olim).  Lane r < WROWS counts
        // row r from the rows' masks; one warp reduction per value.  The row
        // that holds a boundary is split with one ballot: lane j takes bit j
        // when its rank in the run lies below the boundary.
        const uint32_t zlim = ((b.x + zs + CHUNK) & ~(uint32_t)(CHUNK - 1)) - b.x;
        const uint32_t olim = ((b.y + ob0 + CHUNK) & ~(uint32_t)(CHUNK - 1)) - b.y;
        __syncwarp();
        const bool row = lane < (uint32_t)WROWS;
        const uint2 rw = row ? myrow[lane] : make_uint2(0u, 0u);
        const uint32_t omr = rw.x, nzm = rw.y;
        const uint32_t zmr = row ? ~omr : 0u;
        const uint32_t zc = __popc(zmr), oc = __popc(omr);
        uint32_t zpre = zc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t q = __shfl_up_sync(0xffffffffu, zpre, o);
          if (lane >= (uint32_t)o) zpre += q;
        }
        zpre -= zc;                                 // zeros of the chunk before row `lane`
        const uint32_t zrow = zs + zpre;            // level-wide zero rank of the row's first zero
        const uint32_t orow = ob0 + 32u * lane - zpre;  // and one rank of its first one
        const uint32_t nzz = nzm & zmr, nzo = nzm & omr;
        uint32_t t0 = __popc(nzz), t1 = __popc(nzo);
        uint32_t a0 = zlim >= zrow + zc ? t0 : 0u, a1 = olim >= orow + oc ? t1 : 0u;
        const uint32_t zx = __ballot_sync(0xffffffffu, zlim > zrow && zlim < zrow + zc);
        const uint32_t ox = __ballot_sync(0xffffffffu, olim > orow && olim < orow + oc);
        t0 = __reduce_add_sync(0xffffffffu, t0);
        t1 = __reduce_add_sync(0xffffffffu, t1);
        a0 = __reduce_add_sync(0xffffffffu, a0);
        a1 = __reduce_add_sync(0xffffffffu, a1);
        if (zx) {
          const int sr = __ffs(zx) - 1;
          const uint32_t m = __shfl_sync(0xffffffffu, zmr, sr), nm = __shfl_sync(0xffffffffu, nzz, sr);
          const uint32_t q = __shfl_sync(0xffffffffu, zlim - zrow, sr);
          a0 += __popc(__ballot_sync(0xffffffffu, ((nm >> lane) & 1u) && __popc(m & ltmask) < q));
        }
        if (ox) {
          const int sr = __ffs(ox) - 1;
          const uint32_t m = __shfl_sync(0xffffffffu, omr, sr), nm = __shfl_sync(0xffffffffu, nzo, sr);
          const uint32_t q = __shfl_sync(0xffffffffu, olim - orow, sr);
          a1 += __popc(__ballot_sync(0xffffffffu, ((nm >> lane) & 1u) && __popc(m & ltmask) < q));
        }
        const uint32_t k0 = (b.x + zs) >> LOG_CHUNK, k1 = (b.y + ob0) >> LOG_CHUNK;
        if (lane < 4) {  // lanes 0, 1: the zero run's two destination chunks; 2, 3: the one run's
          const uint32_t v = lane == 0 ? a0 : lane == 1 ? t0 - a0 : lane == 2 ? a1 : t1 - a1;
          if (v) atomicAdd(&chunkcnt_next[(lane < 2 ? k0 : k1) + (lane & 1u)], v);
        }
        if (EMIT_NODES && lane < 2) (lane ? nc1 : nc0)[c] = lane ? t1 : t0;
      }
    } else {
      // ---- general path: a node boundary inside the chunk, or its last chunk
      Slot2 tiles_s, nodes_s;
#pragma unroll 1
      for (int r = 0; r < WROWS; ++r) {
        const uint32_t k = r * 32 + lane;
        const bool valid = k < cvalid;
        const T x = wt[k];
        const bool one = valid && ((uint32_t)x & m1);
        const uint32_t om = __ballot_sync(0xffffffffu, one);
        const uint32_t zm = __ballot_sync(0xffffffffu, valid && !one);
        myrow[r].x = om;  // every lane stores the same word: no branch
        const uint32_t zb = z + __popc(zm & ltmask);
        z += __popc(zm);
        const uint32_t p = prefix_of(x, pshift, pmask);
        const uint32_t plo = __shfl_sync(0xffffffffu, p, 0);
        uint2 bb;
        if (__ballot_sync(0xffffffffu, valid && p != plo) == 0) {
          if (plo != cache_p) {
            cache_p = plo;
            cache_b = base_lvl[plo];
          }
          bb = cache_b;
        } else {
          bb = base_lvl[p];
        }
        const uint32_t d = one ? bb.y + (i0 + k - zb) : bb.x + zb;
        const bool ok = valid && d < n32;
        if (ok) dst[d] = x;
        bad |= valid && !ok;
        if (EMIT_TILES) {
          const bool nb0 = ok && !((uint32_t)x & mnext);
          slot2_count(tiles_s, nb0, d >> LOG_CHUNK, chunkcnt_next, lane);
          if (EMIT_NODES) slot2_count(nodes_s, nb0, 2 * p + (one ? 1u : 0u), znext, lane);
        }
      }
      if (EMIT_TILES) {
        slot2_flush(tiles_s, chunkcnt_next, lane);
        if (EMIT_NODES) slot2_flush(nodes_s, znext, lane);
      }
      if (EMIT_NODES && lane < 2) (lane ? nc1 : nc0)[c] = 0u;  // counted by the atomics above
    }
    if (SCATTER && __any_sync(0xffffffffu, bad) && lane == 0) atomicCAS(err, 0u, (uint32_t)DERR_BAD_INDEX);
    __syncwarp();

    // the chunk's bits: word j covers global bits [g + 32 j, g + 32 j + 32)
    const uint64_t g = bit_off + cbase;
    const uint32_t g0 = (uint32_t)(g & 31);
    const uint64_t G = g >> 5;
    if (g0 == 0 && cvalid == CHUNK) {  // whole words of this chunk only
      if (lane < (uint32_t)WROWS) bits32[G + lane] = myrow[lane].x;
    } else if (lane <= (uint32_t)WROWS && !(g0 == 0 && lane == (uint32_t)WROWS)) {
      const uint32_t curw = lane < (uint32_t)WROWS ? myrow[lane].x : 0u;
      const uint32_t prev = lane ? myrow[lane - 1].x : 0u;
      const uint32_t val = g0 ? ((curw << g0) | (prev >> (32 - g0))) : curw;
      const uint64_t wlo = (G + lane) * 32;
      if (wlo < g + cvalid) {
        const bool full = (wlo >= g) && (wlo + 32 <= g + cvalid);
        if (full) bits32[G + lane] = val;
        else if (val) atomicOr(&bits32[G + lane], val);
      }
    }
    __syncwarp();
  }
    slot = slot + 1 == LV_STAGES ? 0 : slot + 1;
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
                         (int)LvShape<T>::template smem<SC>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, level_kernel<T, SC, EN, ET>, LV_THREADS,
                                                  LvShape<T>::template smem<SC>());
    if (per_sm <= 0) per_sm = 1;
  }
  const uint64_t tiles = (n + LvShape<T>::TILE - 1) / LvShape<T>::TILE;
  return (int)std::min<uint64_t>(tiles, (uint64_t)per_sm * sm_count());
}

// Three exclusive scans in one single-pass launch (decoupled look-back, one
// status word array per field; warps 0-2 run the three look-backs side by
// side): after a pass, the next level's chunk zero counts and the two
// per-chunk node counts.  Every prefix stays below n < 2^32.  The arrays are
// 16-byte aligned (per-level strides are whole vectors), so a thread moves
// its 8 items of a field as two 16-byte vectors.
constexpr int S3_THREADS = 256;
constexpr int S3_IPT = 8;
constexpr int S3_TILE = S3_THREADS * S3_IPT;

__global__ void __launch_bounds__(S3_THREADS)
    scan3_kernel(const uint32_t* __restrict__ in0, const uint32_t* __restrict__ in1,
                 const uint32_t* __restrict__ in2, uint32_t* __restrict__ out0, uint32_t* __restrict__ out1,
                 uint32_t* __restrict__ out2, uint64_t n, uint64_t* status, uint64_t sstride, uint32_t* counter,
                 uint32_t* err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_wsum[3][S3_THREADS / 32];
  __shared__ uint32_t s_prefix[3];
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t base = (uint64_t)tile * S3_TILE + (uint64_t)threadIdx.x * S3_IPT;
  const uint32_t* const in[3] = {in0, in1, in2};
  uint32_t v[3][S3_IPT], sum[3], incl[3];
  const bool whole = base + S3_IPT <= n;  // the thread's items as two 16-byte vectors
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    sum[f] = 0;
    if (whole) {
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(in[f] + base));
      const uint4 b = __ldg(reinterpret_cast<const uint4*>(in[f] + base) + 1);
      v[f][0] = a.x; v[f][1] = a.y; v[f][2] = a.z; v[f][3] = a.w;
      v[f][4] = b.x; v[f][5] = b.y; v[f][6] = b.z; v[f][7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < S3_IPT; ++k) v[f][k] = base + k < n ? in[f][base + k] : 0u;
    }
#pragma unroll
    for (int k = 0; k < S3_IPT; ++k) sum[f] += v[f][k];
    incl[f] = sum[f];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl[f], o);
      if (lane >= (uint32_t)o) incl[f] += t;
    }
    if (lane == 31) s_wsum[f][warp] = incl[f];
  }
  __syncthreads();
  if (warp < 3) {
    // warp f: the scan of field f's warp sums, then its look-back
    const uint32_t f = warp;
    const uint32_t w = lane < S3_THREADS / 32 ? s_wsum[f][lane] : 0u;
    uint32_t winc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, winc, o);
      if (lane >= (uint32_t)o) winc += t;
    }
    if (lane < S3_THREADS / 32) s_wsum[f][lane] = winc - w;
    const uint32_t total = __shfl_sync(0xffffffffu, winc, S3_THREADS / 32 - 1);
    uint64_t* st = status + f * sstride;
    uint32_t prefix = 0;
    if (tile == 0) {
      if (lane == 0) lb_publish(st, tile, LB_FLAG_INC, total);
    } else {
      if (lane == 0) lb_publish(st, tile, LB_FLAG_AGG, total);
      prefix = (uint32_t)lb_lookback_warp(st, tile, err);
      if (lane == 0) lb_publish(st, tile, LB_FLAG_INC, (uint64_t)prefix + total);
    }
    if (lane == 0) s_prefix[f] = prefix;
  }
  __syncthreads();
  uint32_t* const out[3] = {out0, out1, out2};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    uint32_t run = s_prefix[f] + s_wsum[f][warp] + incl[f] - sum[f];
    uint32_t o[S3_IPT];
#pragma unroll
    for (int k = 0; k < S3_IPT; ++k) {
      o[k] = run;
      run += v[f][k];
    }
    if (whole) {
      reinterpret_cast<uint4*>(out[f] + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
      reinterpret_cast<uint4*>(out[f] + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
    } else {
#pragma unroll
      for (int k = 0; k < S3_IPT; ++k)
        if (base + k < n) out[f][base + k] = o[k];
    }
  }
}

static int scan3_u32(const uint32_t* in0, const uint32_t* in1, const uint32_t* in2, uint32_t* out0, uint32_t* out1,
                     uint32_t* out2, uint64_t n, DevBuf& scratch, uint32_t* d_err, cudaStream_t s) {
  if (n == 0) return WTG_OK;
  const uint64_t tiles = (n + S3_TILE - 1) / S3_TILE;
  const size_t bytes = (3 * tiles + 1) * sizeof(uint64_t);
  int rc = scratch.ensure(bytes, s);
  if (rc) return rc;
  WTG_CK(cudaMemsetAsync(scratch.p, 0, bytes, s));
  prof_begin(PROF_TABLES, s);
  scan3_kernel<<<(unsigned)tiles, S3_THREADS, 0, s>>>(in0, in1, in2, out0, out1, out2, n,
                                                       scratch.as<uint64_t>() + 1, tiles, scratch.as<uint32_t>(),
                                                       d_err);
  prof_end(PROF_TABLES, s);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

// Node sizes of level l+1 from the per-chunk counts of the pass over level l:
// the chunks lying inside node p are [ceil(C(p)/512), floor(C(p+1)/512)), and
// the exclusive scans S0, S1 of their counts (zeros of 2p, of 2p+1) give
// their sums as S[end] - S[begin].  The chunks across node boundaries added
// theirs with atomics during the pass.
__global__ void node_sum_kernel(const uint32_t* __restrict__ Cl, uint64_t cnt, uint64_t n,
                                const uint32_t* __restrict__ S0, const uint32_t* __restrict__ S1,
                                uint32_t* __restrict__ znext) {
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < cnt; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = ((uint64_t)Cl[p] + CHUNK - 1) / CHUNK;
    const uint64_t e = (p + 1 < cnt ? (uint64_t)Cl[p + 1] : n) / CHUNK;
    if (e > b) {
      znext[2 * p] += S0[e] - S0[b];
      znext[2 * p + 1] += S1[e] - S1[b];
    }
  }
}

struct LevelArgs {
  const void* src;
  void* dst;
  uint64_t n;
  int L, level;
  const uint2* base_lvl;
  uint32_t* bits32;
  uint64_t bit_off;
  const uint32_t* chunkpre;
  uint32_t* chunkcnt_next;
  uint32_t *nc0, *nc1;  // per chunk: counts of the next level's two nodes (emit_nodes)
  uint32_t* znext;
  uint32_t* err;
  uint32_t* chunkcnt_self;
  bool scatter, emit_nodes, emit_tiles;
};

template <typename T, bool SC, bool EN, bool ET>
static void launch_level_v(const LevelArgs& a, cudaStream_t st) {
  const int bulk_ok = ((uintptr_t)a.src % 16) == 0;
  const size_t shm = LvShape<T>::template smem<SC>();
  level_kernel<T, SC, EN, ET><<<level_grid<T, SC, EN, ET>(a.n), LV_THREADS, shm, st>>>(
      (const T*)a.src, (T*)a.dst, a.n, a.L, a.level, a.base_lvl, a.bits32, a.bit_off, a.chunkpre,
      a.chunkcnt_next, a.nc0, a.nc1, a.znext, a.err, bulk_ok, a.chunkcnt_self);
}

template <typename T>
static void launch_level(const LevelArgs& a, cudaStream_t st) {
  if (a.scatter && a.emit_nodes) launch_level_v<T, true, true, true>(a, st);
  else if (a.scatter && a.emit_tiles) launch_level_v<T, true, false, true>(a, st);
  else if (a.scatter) launch_level_v<T, true, false, false>(a, st);
  else launch_level_v<T, false, false, false>(a, st);
}

template <typename T>
static void launch_prepass(const void* s, uint64_t n, int L, int K, uint64_t c_begin, uint64_t c_end,
                           uint32_t* tilecnt, uint32_t* hist, cudaStream_t st) {
  const uint64_t chunks = c_end - c_begin;
  unsigned grid = (unsigned)std::min<uint64_t>((chunks + 7) / 8, (uint64_t)sm_count() * 8);
  if (grid == 0) grid = 1;
  const int vec_ok = ((uintptr_t)s % 16) == 0;
  prepass_kernel<T><<<grid, LV_THREADS, 0, st>>>((const T*)s, n, L, K, vec_ok, c_begin, c_end, tilecnt, hist);
}

#define WTG_DISPATCH(eb, fn, ...)                       \
  switch (eb) {                                         \
    case 1: fn<uint8_t>(__VA_ARGS__); break;            \
    case 2: fn<uint16_t>(__VA_ARGS__); break;           \
    case 4: fn<uint32_t>(__VA_ARGS__); break;           \
    default: fn<uint64_t>(__VA_ARGS__); break;          \
  }

static uint64_t tile_elems(int) { return CHUNK; }  // counts are kept per 512-symbol chunk

// host memory the device copies to and from without staging (page-locked or
// registered)
bool host_page_locked(const void* p) {
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
    cudaGetLastError();  // clear the query's error
    return false;
  }
  return pa.type == cudaMemoryTypeHost;
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
  t.lvl_args_ok = false;
  t.node_tab_ok = false;
  ++t.gen;
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
  // [L + 1][tst] counts, then [L][tst] prefixes (kept per level:
  // the rank/select pass reads them all)
  // per-level stride: tiles + 1 entries, rounded up to whole 16-byte vectors
  const uint64_t tst = (tiles + 4) & ~3ull;
  if ((rc = t.status.ensure((2 * (uint64_t)L + 1) * tst * sizeof(uint32_t), s))) return rc;
  uint32_t* tilecnt = t.status.as<uint32_t>();
  uint32_t* tilepre_all = tilecnt + ((uint64_t)L + 1) * tst;
  if (n) WTG_CK(cudaMemsetAsync(tilecnt, 0, (uint64_t)L * tst * sizeof(uint32_t), s));

  if (n) {
    const uint64_t nchunks = (n + CHUNK - 1) / CHUNK;
    prof_begin(PROF_HIST, s);
    if (t.in_pieces > 0) {
      // each piece of the input is counted once its copy has landed; the
      // passes after the pre-pass see the whole input
      for (int i = 0; i < t.in_pieces; ++i) {
        const uint64_t c0 = std::min<uint64_t>(nchunks, (uint64_t)i * t.in_piece_chunks);
        const uint64_t c1 = std::min<uint64_t>(nchunks, c0 + t.in_piece_chunks);
        WTG_CK(cudaStreamWaitEvent(s, t.in_ev[i], 0));
        if (c1 > c0) {
          WTG_DISPATCH(eb, launch_prepass, d_seq, n, L, K, c0, c1, tilecnt, S, s);
          count_launch();
          WTG_CK(cudaGetLastError());
        }
      }
    } else {
      WTG_DISPATCH(eb, launch_prepass, d_seq, n, L, K, 0, nchunks, tilecnt, S, s);
      count_launch();
      WTG_CK(cudaGetLastError());
    }
    prof_end(PROF_HIST, s);
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

  // per-chunk node counts of a pass and their scans: [nc0 | nc1 | S0 | S1]
  if (n && L > K) {
    if ((rc = t.nodecnt.ensure(4 * tst * sizeof(uint32_t), s))) return rc;
    WTG_CK(cudaMemsetAsync(t.nodecnt.p, 0, 2 * tst * sizeof(uint32_t), s));
  }

  // level passes; each scattering pass feeds the next level's chunk counts
  // and (from level K on) its node tables.  With n % 512 == 0 the chunk
  // counts of every level also give the rank/select pass its prefixes.
  const bool rs_from_levels = flags && n > 0 && (n % CHUNK) == 0;
  // When the rank table goes to page-locked host memory during the build,
  // the rank/select pass runs level by level after each level pass, and each
  // level's rank entries are copied while the later levels are built (a copy
  // to pageable memory would hold the host until it ends); otherwise it is
  // one launch over all levels after the last pass.
  const bool rs_by_level = rs_from_levels && t.host_rank && (flags & WTG_RANK) && host_page_locked(t.host_rank);
  uint64_t* lvl_zb = nullptr;
  if (rs_from_levels) {
    if ((rc = t.scratch.ensure(((uint64_t)L + 1) * sizeof(uint64_t), s))) return rc;
    lvl_zb = t.scratch.as<uint64_t>();
    if ((rc = bv_levels_begin(t.bv, t.bits.as<uint64_t>(), n, L, flags, s))) return rc;
  }
  const uint64_t rank_words_per_level = 2 * (n / CHUNK);  // rank entries of one level when n % 512 == 0
  auto copy_rank_level = [&](int l) -> int {
    const uint64_t off = (uint64_t)l * rank_words_per_level;
    WTG_CK(cudaEventRecord(t.copy_ev, s));
    WTG_CK(cudaStreamWaitEvent(t.copy_stream, t.copy_ev, 0));
    WTG_CK(cudaMemcpyAsync(t.host_rank + off, t.bv.rank.as<uint64_t>() + off, rank_words_per_level * 8,
                           cudaMemcpyDeviceToHost, t.copy_stream));
    return WTG_OK;
  };
  if (n) {
    if (L > 1) {
      if ((rc = t.lvl[0].ensure(n * eb + 16, s))) return rc;
      if ((rc = t.lvl[1].ensure(n * eb + 16, s))) return rc;
    }
    const void* src = d_seq;
    bool pre_ready = false;  // the level's chunk prefixes were scanned with the previous pass's counts
    for (int l = 0; l < L; ++l) {
      LevelArgs a{};
      a.scatter = l < L - 1;
      a.emit_tiles = l + 1 <= L - 2;
      a.emit_nodes = a.emit_tiles && (l + 1 >= K);
      a.src = src;
      a.dst = a.scatter ? t.lvl[l & 1].p : nullptr;
      a.n = n;
      a.L = L;
      a.level = l;
      a.base_lvl = base + ((1ull << l) - 1);
      a.bits32 = t.bits.as<uint32_t>();
      a.bit_off = (uint64_t)l * n;
      uint32_t* tilepre = tilepre_all + (uint64_t)l * tst;
      a.chunkpre = tilepre;
      a.chunkcnt_next = tilecnt + (uint64_t)(l + 1) * tst;
      a.chunkcnt_self = (!a.scatter && rs_from_levels) ? tilecnt + (uint64_t)l * tst : nullptr;
      a.znext = Z + ((1ull << (l + 1)) - 1);
      a.nc0 = a.emit_nodes ? t.nodecnt.as<uint32_t>() : nullptr;
      a.nc1 = a.emit_nodes ? a.nc0 + tst : nullptr;
      a.err = d_err;
      if (a.scatter && !pre_ready)
        if ((rc = scan_exclusive_u32(tilecnt + (uint64_t)l * tst, tilepre, tiles, t.scan_tmp, d_err, s)))
          return rc;
      pre_ready = false;
      prof_begin(a.scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      WTG_DISPATCH(eb, launch_level, a, s);
      prof_end(a.scatter ? PROF_LEVEL : PROF_LEVEL_LAST, s);
      count_launch();
      WTG_CK(cudaGetLastError());
      if (a.emit_nodes) {
        // the next level's chunk prefixes and the in-node chunks' counts in
        // one scan, then one sum per node of level l
        uint32_t* S0 = a.nc0 + 2 * tst;
        uint32_t* S1 = a.nc0 + 3 * tst;
        if ((rc = scan3_u32(a.chunkcnt_next, a.nc0, a.nc1, tilepre_all + (uint64_t)(l + 1) * tst, S0, S1,
                            tiles + 1, t.scan_tmp, d_err, s)))
          return rc;
        pre_ready = true;
        const uint64_t cnt = 1ull << l;
        unsigned grid = (unsigned)std::min<uint64_t>((cnt + 255) / 256, 2048);
        prof_begin(PROF_TABLES, s);
        node_sum_kernel<<<grid, 256, 0, s>>>(C + cnt - 1, cnt, n, S0, S1, a.znext);
        prof_end(PROF_TABLES, s);
        count_launch();
        WTG_CK(cudaGetLastError());
      }
      src = a.dst;
      if (t.host_bits) {
        // words holding only bits of levels <= l are final now; the word
        // shared with level l + 1 goes with the next level
        const uint64_t w_lo = ((uint64_t)l * n) >> 6;
        const uint64_t w_hi = (l == L - 1) ? t.bit_words : (((uint64_t)l + 1) * n) >> 6;
        if (w_hi > w_lo) {
          WTG_CK(cudaEventRecord(t.copy_ev, s));
          WTG_CK(cudaStreamWaitEvent(t.copy_stream, t.copy_ev, 0));
          WTG_CK(cudaMemcpyAsync(t.host_bits + w_lo, t.bits.as<uint64_t>() + w_lo, (w_hi - w_lo) * 8,
                                 cudaMemcpyDeviceToHost, t.copy_stream));
        }
      }
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
      // a scattering level's chunk prefixes were scanned before its pass
      if (rs_by_level && l < L - 1) {
        if ((rc = bv_levels_pass(t.bv, n, l, l + 1, tilecnt, tilepre_all, tst, tiles, lvl_zb, s))) return rc;
        if ((rc = copy_rank_level(l))) return rc;
      }
    }
  }

  // rank / select over the concatenated bitvector
  t.bv.rank_done = (t.host_rank && (flags & WTG_RANK)) ? t.rank_ev : nullptr;
  if (rs_from_levels) {
    uint32_t* last_cnt = tilecnt + (uint64_t)(L - 1) * tst;
    uint32_t* last_pre = tilepre_all + (uint64_t)(L - 1) * tst;
    if ((rc = scan_exclusive_u32(last_cnt, last_pre, tiles, t.scan_tmp, d_err, s))) return rc;
    if ((rc = bv_levels_pass(t.bv, n, rs_by_level ? L - 1 : 0, L, tilecnt, tilepre_all, tst, tiles, lvl_zb, s)))
      return rc;
    if (rs_by_level && (rc = copy_rank_level(L - 1))) return rc;
    if ((rc = bv_levels_end(t.bv, L, lvl_zb, d_err, s))) return rc;
  } else if (flags) {
    if ((rc = bv_build(t.bv, t.bits.as<uint64_t>(), n * (uint64_t)L, flags, d_err, s))) return rc;
  }
  if (t.bv.rank_done) {
    // the rank table (level by level: the rest, its final pair) was complete
    // before the select finishing kernels started; its copy runs beside them
    const uint64_t size = n * (uint64_t)L;
    const uint64_t cap = (size + 63) / 64 * 64;
    const uint64_t rank_words = size ? ((cap >> 9) + 1) * 2 : 2;
    const uint64_t from = rs_by_level ? rank_words - 2 : 0;
    WTG_CK(cudaStreamWaitEvent(t.copy_stream, t.bv.rank_done, 0));
    WTG_CK(cudaMemcpyAsync(t.host_rank + from, t.bv.rank.as<uint64_t>() + from, (rank_words - from) * 8,
                           cudaMemcpyDeviceToHost, t.copy_stream));
    t.bv.rank_done = nullptr;
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
  if (t.copy_stream) {
    cudaStreamSynchronize(t.copy_stream);
    cudaStreamDestroy(t.copy_stream);
    t.copy_stream = nullptr;
  }
  if (t.copy_ev) cudaEventDestroy(t.copy_ev);
  if (t.rank_ev) cudaEventDestroy(t.rank_ev);
  t.copy_ev = t.rank_ev = nullptr;
  if (t.in_stream) {
    cudaStreamSynchronize(t.in_stream);
    cudaStreamDestroy(t.in_stream);
    t.in_stream = nullptr;
  }
  for (cudaEvent_t& e : t.in_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  t.in_pieces = 0;
  lsel_detach_all(t);
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
  t.lvl_args.release(s);
  t.lvl_args_ok = false;
  t.fm_paths.release(s);
  t.node_tab.release(s);
  t.node_tab_ok = false;
  t.scratch.release(s);
  t.nodes.release(s);
  t.nodecnt.release(s);
  t.qbuf.release(s);
  t.qout.release(s);
  bv_release(t.bv, s);
}

}  // namespace wtg
