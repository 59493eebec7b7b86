// wtg_batch.cu -- batched builds: many independent texts, each with its own
// wavelet tree (level bitvector of L <= 4 levels), rank_support_v<1> and
// select_support_mcl<1>/<0>, all in one persistent launch.
//
// The reference builds one sequence per WT() call (levelWT/WT.C:43-227,
// driven by levelWT/WTTime.C:78-103); a batch there is a loop of calls.  Here
// one persistent kernel pulls texts from a device queue, largest first, and
// one CTA builds a whole text -- the data of a text (at most a few MB) stays
// in L2 across the CTA's passes:
//   H  symbol histogram -> per level l and node key k (the top l bits) the
//      bit position where that node's bits start: l*n + (symbols whose key
//      is below k).  Level l is the text stably sorted by the top l bits
//      (levelWT/WT.C:118-190), so a symbol's bit at level l lands at
//      start(l, key) + (symbols of the same key before it): every level is
//      written from one read of the text, no level-by-level passes.
//   W  per chunk, warp slices count their symbols per (level, key), a block
//      scan gives each slice its run offsets, and each warp appends its
//      compacted bits to those runs (ballot + in-warp compaction).
//   R  one pass over the text's bits: rank_support_v table (the reference
//      layout and final-superblock rule) and the select sample marks.
//   S  select_support_mcl per polarity: long/mini choice, widths, pool
//      offsets (block scan), mini blocks from the samples, long blocks by
//      rank-table search, m_superblock packing.
// Every output has the layout of the single-sequence build.  The pool region
// of each text is sized by a bound that holds for any input (see plan), so
// the layout is fixed by the text lengths alone.  The launch shape (threads
// per CTA, symbols per thread per chunk) is picked by timing the candidates
// on the batch itself, and the memsets plus the launch are captured in a
// CUDA graph that later runs replay.
#include <algorithm>
#include <numeric>
#include <vector>

#include "wtg_internal.cuh"
#include "wtg_select.cuh"

namespace wtg {

WTG_WAIT_LIMIT_SETTER(batch)

constexpr int BATCH_LMAX = 4;
constexpr int BATCH_SLOTS = (1 << BATCH_LMAX) - 1;  // (level, key) pairs
constexpr uint32_t BATCH_INVALID = 0xFFFFFFFFu;
constexpr int BATCH_MAX_CHUNK = 8192;  // THREADS * IPT of every launch shape

struct BatchArgs {
  const uint8_t* sym;     // concatenated texts
  const uint64_t* so;     // symbol offset of each text, T + 1
  const uint32_t* order;  // texts by decreasing length
  uint64_t T;
  int L;
  uint32_t flags;
  uint64_t* bits;
  const uint64_t* bo;  // word offset of each text's bits
  uint64_t* rank;
  const uint64_t* ro;
  uint32_t* samples;
  const uint64_t* sao;
  uint64_t* marks;  // starts1 | starts0 | ends1 | ends0, nsbc entries each
  const uint64_t* mo;
  uint64_t* desc[2];
  const uint64_t* deo;
  uint64_t* sbw[2];
  const uint64_t* sbo;
  uint64_t* pool[2];
  const uint64_t* poo[2];  // T + 1 entries: region bounds
  uint64_t* info;          // 8 per text: m1, m0, last1, last0, pool1, pool0, nlong1, nlong0
  uint32_t* queue;
  uint32_t* err;
};

template <int THREADS>
struct BatchSmem {
  static constexpr int NW = THREADS / 32;
  uint32_t item;
  uint32_t hist[1 << BATCH_LMAX];
  uint64_t base[BATCH_SLOTS];
  uint64_t carry[BATCH_SLOTS];
  uint32_t cnt[NW][BATCH_SLOTS];
  uint64_t start[NW][BATCH_SLOTS];
  uint64_t wsum[NW];
  uint64_t run;
  unsigned long long last[2];
  uint32_t nlong;
  uint64_t ent[NW][64];
  // phase W: two staging buffers for chunks of up to BATCH_MAX_CHUNK symbols
  // (plus the text's offset from a 16-byte boundary), filled by cp.async.bulk
  alignas(16) uint8_t stage[2][BATCH_MAX_CHUNK + 32];
  alignas(8) uint64_t bar[2];
};

__device__ __forceinline__ uint64_t batch_logn(uint64_t size) {
  const uint64_t cap = (size + 63) / 64 * 64;
  return hi64(cap) + 1;
}

// block-wide exclusive scan of one u64 per thread; returns the prefix and
// the block total through *total
template <int THREADS>
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, BatchSmem<THREADS>& sm, uint64_t* total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) sm.wsum[warp] = inc;
  __syncthreads();
  uint64_t before = 0, all = 0;
  for (int w = 0; w < BatchSmem<THREADS>::NW; ++w) {
    const uint64_t x = sm.wsum[w];
    before += (w < (int)warp) ? x : 0;
    all += x;
  }
  __syncthreads();
  *total = all;
  return before + inc - v;
}

// k-th (0-based) arg of a bitvector, found by binary search over the rank
// table between superblocks lo and hi, then popcounts of at most 8 words
__device__ __forceinline__ uint64_t batch_select_by_rank(int t_b, const uint64_t* __restrict__ words,
                                                         const uint64_t* __restrict__ rank, uint64_t W,
                                                         uint64_t tailmask, uint64_t lo, uint64_t hi, uint64_t k,
                                                         uint32_t* err) {
  const uint64_t last_sb = W >> 3;  // superblock entries 0 .. W/8
  if (hi > last_sb) hi = last_sb;
  if (lo > hi) lo = hi;
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) >> 1;
    const uint64_t r = rank[2 * mid];
    if ((t_b ? r : 512 * mid - r) <= k) lo = mid;
    else hi = mid - 1;
  }
  const uint64_t r = rank[2 * lo];
  uint64_t rem = k - (t_b ? r : 512 * lo - r);
  for (uint64_t wi = 8 * lo; wi < 8 * lo + 8 && wi < W; ++wi) {
    uint64_t x = __ldcg(words + wi);
    if (!t_b) x = ~x;
    if (wi == W - 1) x &= tailmask;
    const uint32_t c = __popcll(x);
    if (rem < c) return (wi << 6) + sel64(x, (uint32_t)rem + 1);
    rem -= c;
  }
  atomicCAS(err, 0u, (uint32_t)DERR_SELECT_OVERFLOW);
  return 0;
}

// Run of (level l, key k) in a row: the valid lanes whose symbol's bits
// above level l spell k (planes P[j] = ballot of bit j, V = valid lanes)
template <int LL>
__device__ __forceinline__ uint32_t batch_run_mask(const uint32_t* P, uint32_t V, int l, uint32_t k) {
  uint32_t m = V;
#pragma unroll
  for (int j = LL - 1; j >= 0; --j)
    if (j >= LL - l) m &= ((k >> (j - (LL - l))) & 1u) ? P[j] : ~P[j];
  return m;
}

// The level bits of one text: every (level, key) run is one contiguous bit
// range of its level, so per chunk of THREADS * IPT symbols a warp counts
// its rows' members of every run (one ballot per bit plane and row; run
// masks from logic ops), the block places the warps' pieces, and each warp
// appends its pieces: level 0's run is the valid lanes, a prefix of the row,
// so its bits are the plane itself; deeper runs compact the plane to the
// run with one OR-reduction of 1 << rank.  All runs are carried through the
// rows together, their words written whole or, at a run's first and last
// word (shared with the neighbouring pieces), ORed.
template <int THREADS, int IPT, int LL>
__device__ void batch_write_bits(const uint8_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ bits,
                                 BatchSmem<THREADS>& sm, uint32_t& phases, uint32_t* err) {
  constexpr int NW = THREADS / 32;
  constexpr int NS = (1 << LL) - 1;  // runs: (level, key) slots
  constexpr uint64_t CH = (uint64_t)THREADS * IPT;
  static_assert(CH <= BATCH_MAX_CHUNK, "chunk larger than the staging buffers");
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t vmask = (1u << LL) - 1, lt = (1u << lane) - 1;
  // chunks are staged by thread 0 one ahead: from the 16-byte boundary at
  // or below the chunk (the input has 16 bytes of padding after the last
  // text, so the rounded-up tail stays inside it)
  const uint32_t off = (uint32_t)((uintptr_t)in & 15u);
  auto stage_chunk = [&](uint64_t c, int buf) {
    const uint64_t cnt = min(CH, n - c);
    const uint32_t bytes = (uint32_t)((off + cnt + 15) & ~15ull);
    fence_proxy_async_smem();
    mbar_expect_tx(&sm.bar[buf], bytes);
    bulk_g2s(sm.stage[buf], in + c - off, bytes, &sm.bar[buf]);
  };
  int cur = 0;
  if (tid == 0 && n) stage_chunk(0, 0);
  for (uint64_t c0 = 0; c0 < n; c0 += CH, cur ^= 1) {
    if (tid == 0 && c0 + CH < n) stage_chunk(c0 + CH, cur ^ 1);  // its last readers passed the previous barrier
    mbar_wait(&sm.bar[cur], (phases >> cur) & 1u, err);
    phases ^= 1u << cur;
    const uint8_t* const st = sm.stage[cur] + off;
    const uint64_t s0 = c0 + (uint64_t)warp * 32 * IPT;
    uint32_t v[IPT];
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const uint64_t i = s0 + 32 * r + lane;
      v[r] = i < n ? (st[i - c0] & vmask) : BATCH_INVALID;
    }
    uint32_t cnt[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) cnt[q] = 0;
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const bool valid = v[r] != BATCH_INVALID;
      uint32_t P[LL];
#pragma unroll
      for (int j = 0; j < LL; ++j) P[j] = __ballot_sync(0xffffffffu, valid && ((v[r] >> j) & 1u));
      const uint32_t V = __ballot_sync(0xffffffffu, valid);
#pragma unroll
      for (int l = 0, q = 0; l < LL; ++l)
#pragma unroll
        for (uint32_t k = 0; k < (1u << l); ++k, ++q) cnt[q] += __popc(batch_run_mask<LL>(P, V, l, k));
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NS; ++q) sm.cnt[warp][q] = cnt[q];
    }
    __syncthreads();
    if (tid < (uint32_t)NS) {
      uint64_t run = sm.carry[tid];
      for (int w = 0; w < NW; ++w) {
        sm.start[w][tid] = run;
        run += sm.cnt[w][tid];
      }
      sm.carry[tid] = run;
    }
    __syncthreads();
    uint64_t acc[NS], word[NS];
    uint32_t fill[NS];
    bool shared_word[NS];
    const uint64_t lvl0_dest = sm.base[0] + sm.start[warp][0];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      const uint64_t dest = sm.base[q] + sm.start[warp][q];
      word[q] = dest >> 6;
      fill[q] = (uint32_t)(dest & 63);
      shared_word[q] = fill[q] != 0;  // the first word may hold the previous piece's tail
      acc[q] = 0;
    }
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const bool valid = v[r] != BATCH_INVALID;
      uint32_t P[LL];
#pragma unroll
      for (int j = 0; j < LL; ++j) P[j] = __ballot_sync(0xffffffffu, valid && ((v[r] >> j) & 1u));
      const uint32_t V = __ballot_sync(0xffffffffu, valid);
#pragma unroll
      for (int l = 0, q = 0; l < LL; ++l) {
        const int bs = LL - 1 - l;
#pragma unroll
        for (uint32_t k = 0; k < (1u << l); ++k, ++q) {
          const uint32_t m = batch_run_mask<LL>(P, V, l, k);
          const uint32_t cm = __popc(m);
          if (cm == 0) continue;
          uint32_t comp;
          if (l == 0) {
            // level 0 holds every symbol in order: row r of this warp is the
            // 32-bit word (dest >> 5) + r (dest = its first bit, a multiple
            // of 32); a partial row shares its word with level 1's first bits
            comp = P[bs] & V;
            if (lane == 0) {
              uint32_t* const w32 = reinterpret_cast<uint32_t*>(bits) + (lvl0_dest >> 5) + r;
              if (V == 0xffffffffu) *w32 = comp;
              else if (comp) atomicOr(w32, comp);
            }
            continue;
          } else {
            const uint32_t one = ((m & P[bs]) >> lane) & 1u ? (1u << __popc(m & lt)) : 0u;
            comp = __reduce_or_sync(0xffffffffu, one);
          }
          acc[q] |= (uint64_t)comp << fill[q];
          if (fill[q] + cm >= 64) {
            if (lane == 0 && acc[q]) {
              if (shared_word[q]) atomicOr((unsigned long long*)&bits[word[q]], (unsigned long long)acc[q]);
              else bits[word[q]] = acc[q];
            }
            acc[q] = fill[q] ? ((uint64_t)comp >> (64 - fill[q])) : 0;
            fill[q] = fill[q] + cm - 64;
            ++word[q];
            shared_word[q] = false;
          } else {
            fill[q] += cm;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NS; ++q)
      if (lane == 0 && fill[q] && acc[q]) atomicOr((unsigned long long*)&bits[word[q]], (unsigned long long)acc[q]);
    __syncthreads();
  }
}

template <int THREADS, int IPT>
__device__ void batch_text(const BatchArgs& a, uint64_t t, BatchSmem<THREADS>& sm, uint32_t& phases) {
  constexpr int NW = THREADS / 32;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int L = a.L;
  const uint32_t nbin = 1u << L, vmask = nbin - 1;
  const int nslot = (1 << L) - 1;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint8_t* __restrict__ in = a.sym + a.so[t];
  uint64_t* __restrict__ bits = a.bits + a.bo[t];

  // ---- H: histogram and run starts.  The order of the symbols does not
  // matter here, so each thread reads 16 at a time and counts the low-L-bit
  // values of a 32-bit word bit-sliced (L <= 2) or bytewise (L = 3, 4);
  // bin 0 is what remains.
  if (tid < (1u << BATCH_LMAX)) sm.hist[tid] = 0;
  __syncthreads();
  {
    uint32_t c[1 << BATCH_LMAX];
#pragma unroll
    for (int b = 0; b < (1 << BATCH_LMAX); ++b) c[b] = 0;
    const uint32_t bmask = vmask * 0x01010101u;
    auto count_word = [&](uint32_t w) {  // four symbols
      const uint32_t x = w & bmask;
      if (L == 1) {
        c[1] += __popc(x);
      } else if (L == 2) {
        const uint32_t lo = x & 0x01010101u, hi = (x >> 1) & 0x01010101u, both = __popc(lo & hi);
        c[1] += __popc(lo) - both;
        c[2] += __popc(hi) - both;
        c[3] += both;
      } else {
#pragma unroll
        for (int b = 1; b < (1 << BATCH_LMAX); ++b)
          if ((uint32_t)b < nbin) c[b] += __popc(__vcmpeq4(x, (uint32_t)b * 0x01010101u)) >> 3;
      }
    };
    const uint64_t head = min(n, (uint64_t)((16u - ((uintptr_t)in & 15u)) & 15u));  // bytes before a 16-byte boundary
    const uint64_t nvec = (n - head) / 16;
    const uint64_t rest = head + nvec * 16;
    if (tid < head) count_word(in[tid]);
    if (tid < n - rest) count_word(in[rest + tid]);
    const uint4* vin = reinterpret_cast<const uint4*>(in + head);
    uint64_t q = tid;
    for (; q + THREADS < nvec; q += 2 * THREADS) {
      const uint4 u = __ldg(vin + q), v = __ldg(vin + q + THREADS);
      count_word(u.x); count_word(u.y); count_word(u.z); count_word(u.w);
      count_word(v.x); count_word(v.y); count_word(v.z); count_word(v.w);
    }
    if (q < nvec) {
      const uint4 u = __ldg(vin + q);
      count_word(u.x); count_word(u.y); count_word(u.z); count_word(u.w);
    }
#pragma unroll
    for (int b = 1; b < (1 << BATCH_LMAX); ++b) {
      if ((uint32_t)b >= nbin) continue;
      const uint32_t t = __reduce_add_sync(0xffffffffu, c[b]);
      if (lane == 0 && t) atomicAdd(&sm.hist[b], t);
    }
  }
  __syncthreads();
  if (tid == 0) {
    uint64_t others = 0;
    for (uint32_t b = 1; b < nbin; ++b) others += sm.hist[b];
    sm.hist[0] = (uint32_t)(n - others);
  }
  __syncthreads();
  if (tid < (uint32_t)nslot) {
    int l = 0;
    while ((2 << l) - 1 <= (int)tid) ++l;
    const uint32_t k = tid - ((1u << l) - 1);
    uint64_t below = 0;
    for (uint32_t b = 0; b < nbin; ++b)
      if ((b >> (L - l)) < k) below += sm.hist[b];
    sm.base[tid] = (uint64_t)l * n + below;
    sm.carry[tid] = 0;
  }
  __syncthreads();

  // ---- W: level bits (batch_write_bits, compiled per level count)
  switch (L) {
    case 1: batch_write_bits<THREADS, IPT, 1>(in, n, bits, sm, phases, a.err); break;
    case 2: batch_write_bits<THREADS, IPT, 2>(in, n, bits, sm, phases, a.err); break;
    case 3: batch_write_bits<THREADS, IPT, 3>(in, n, bits, sm, phases, a.err); break;
    default: batch_write_bits<THREADS, IPT, 4>(in, n, bits, sm, phases, a.err); break;
  }
  __syncthreads();

  // ---- R: rank table and select marks
  const uint64_t size = (uint64_t)L * n;
  const uint64_t W = (size + 63) / 64;
  const uint64_t NB = W >> 3;
  const uint64_t r_last = W - 8 * NB;
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  const bool do_rank = (a.flags & (WTG_RANK | WTG_SELECT1 | WTG_SELECT0)) != 0;
  const bool sel1 = a.flags & WTG_SELECT1, sel0 = a.flags & WTG_SELECT0;
  uint64_t* __restrict__ rank = a.rank + a.ro[t];
  uint32_t* __restrict__ samples = a.samples + a.sao[t];
  const uint64_t samp_last = W + 1;
  const uint64_t nsbc = size / 4096 + 2;
  uint64_t* __restrict__ starts1 = a.marks + a.mo[t];
  uint64_t* __restrict__ starts0 = starts1 + nsbc;
  uint64_t* __restrict__ ends1 = starts0 + nsbc;
  uint64_t* __restrict__ ends0 = ends1 + nsbc;
  if (!do_rank) return;
  if (tid == 0) {
    sm.run = 0;
    sm.last[0] = sm.last[1] = 0;
  }
  __syncthreads();
  {
    const uint32_t g8 = lane & 7;
    uint64_t last1 = 0, last0 = 0;
    for (uint64_t w0 = 0; w0 < 8 * (NB + 1); w0 += THREADS) {
      const uint64_t wi = w0 + tid;
      // through L2: the boundary words of phase W were ORed there by atomics,
      // which leave any copy of the line in this SM's L1 unchanged
      uint64_t x = wi < W ? __ldcg(bits + wi) : 0ull;
      if (wi == W - 1) x &= tailmask;
      const uint32_t c = __popcll(x);
      uint32_t inc = c;
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        const uint32_t q = __shfl_up_sync(0xffffffffu, inc, o);
        if (g8 >= (uint32_t)o) inc += q;
      }
      const uint32_t sbt = __shfl_sync(0xffffffffu, inc, (lane & ~7u) + 7);
      // exclusive prefix of the superblock totals within the warp (4 groups)
      const uint32_t t0 = __shfl_sync(0xffffffffu, inc, 7), t1 = __shfl_sync(0xffffffffu, inc, 15),
                     t2 = __shfl_sync(0xffffffffu, inc, 23), t3 = __shfl_sync(0xffffffffu, inc, 31);
      const uint32_t grp = lane >> 3;
      const uint32_t gpre = (grp > 0 ? t0 : 0) + (grp > 1 ? t1 : 0) + (grp > 2 ? t2 : 0);
      if (lane == 0) sm.wsum[warp] = (uint64_t)t0 + t1 + t2 + t3;
      __syncthreads();
      uint64_t wpre = 0, all = 0;
      for (int w = 0; w < NW; ++w) {
        const uint64_t q = sm.wsum[w];
        wpre += (w < (int)warp) ? q : 0;
        all += q;
      }
      const uint64_t sb_before = sm.run + wpre + gpre;
      const uint32_t excl = inc - c;
      const uint64_t b = wi >> 3;
      if (a.flags & WTG_RANK) {
        const uint32_t kmax = (b < NB) ? 7u : (r_last > 1 ? (uint32_t)r_last : 1u);
        uint64_t part = (g8 >= 1 && g8 <= kmax) ? ((uint64_t)excl << (63 - 9 * g8)) : 0ull;
  #pragma unroll
      for (int o = 1; o < 8; o <<= 1) part |= __shfl_xor_sync(0xffffffffu, part, o);
        if (g8 == 0 && b <= NB) {
          rank[2 * b] = sb_before;
          rank[2 * b + 1] = part;
        }
      }
      (void)sbt;
      if (wi < W)
        word_marks(x, c, sb_before + excl, wi, wi == W - 1 ? tailmask : ~0ull, sel1, sel0, samples, samp_last,
                   starts1, starts0, ends1, ends0, last1, last0);
      __syncthreads();
      if (tid == 0) sm.run += all;
      __syncthreads();
    }
    atomicMax(&sm.last[1], (unsigned long long)last_arg_end(bits, last1, W, tailmask, 1));
    atomicMax(&sm.last[0], (unsigned long long)last_arg_end(bits, last0, W, tailmask, 0));
  }
  __syncthreads();
  const uint64_t m1 = sm.run, m0 = size - m1;
  const uint64_t last1 = sm.last[1], last0 = sm.last[0];
  uint64_t* info = a.info + 8 * t;
  if (tid == 0) {
    info[0] = m1;
    info[1] = m0;
    info[2] = last1;
    info[3] = last0;
  }
  __syncthreads();  // every thread has read sm.run before phase S reuses it

  // ---- S: select_support_mcl per polarity
  const uint32_t logn = (uint32_t)batch_logn(size);
  const uint64_t logn4 = (uint64_t)(uint32_t)(logn * logn * logn * logn);
  for (int t_b = 1; t_b >= 0; --t_b) {
    if (!(t_b ? sel1 : sel0)) continue;
    const uint64_t m = t_b ? m1 : m0;
    const uint64_t nsb = (m + 4095) >> 12;
    const uint64_t last = t_b ? last1 : last0;
    const uint64_t* __restrict__ st = t_b ? starts1 : starts0;
    const uint64_t* __restrict__ en = t_b ? ends1 : ends0;
    uint64_t* __restrict__ desc = a.desc[t_b] + a.deo[t];
    uint64_t* __restrict__ pool = a.pool[t_b] + a.poo[t_b][t];
    const uint64_t pool_cap = a.poo[t_b][t + 1] - a.poo[t_b][t];
    if (tid == 0) {
      sm.run = 0;
      sm.nlong = 0;
    }
    __syncthreads();
    for (uint64_t i0 = 0; i0 < nsb; i0 += THREADS) {
      const uint64_t i = i0 + tid;
      uint64_t sz = 0, d = 0;
      if (i < nsb) {
        const uint64_t start = st[i];
        const uint64_t end = (i + 1 < nsb) ? en[i] : last - 1;
        const uint64_t span = end - start;
        const uint64_t lng = span > logn4;
        const uint64_t wdt = lng ? hi64(end) + 1 : hi64(span) + 1;
        d = (lng << 7) | wdt;
        sz = lng ? 64 * wdt : wdt;
        if (lng) atomicAdd(&sm.nlong, 1u);
      }
      uint64_t total;
      const uint64_t off = sm.run + block_excl_scan<THREADS>(sz, sm, &total);
      if (i < nsb) {
        if (off + sz > pool_cap) atomicCAS(a.err, 0u, (uint32_t)DERR_SELECT_OVERFLOW);
        desc[i] = (off << 8) | d;
      }
      __syncthreads();
      if (tid == 0) sm.run += total;
      // fill: warp per superblock of this chunk
      for (uint64_t j = warp; j < (uint64_t)THREADS && i0 + j < nsb; j += NW) {
        const uint64_t si = i0 + j;
        const uint64_t dd = desc[si];
        const uint64_t poff = dd >> 8;
        const uint32_t wdt = (uint32_t)(dd & 127);
        if (poff + ((dd >> 7) & 1 ? 64ull * wdt : wdt) > pool_cap) continue;
        if (!((dd >> 7) & 1)) {
          const uint32_t start = t_b ? samples[64 * si] : samples[samp_last - 64 * si];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t e = lane + 32 * h;
            const uint64_t k = 4096 * si + 64 * (uint64_t)e;
            uint64_t ent = 0;  // entries past the arg count stay zero; their samples do not exist
            if (k < m) {
              const uint32_t sp = t_b ? samples[64 * si + e] : samples[samp_last - (64 * si + e)];
              ent = (uint64_t)(uint32_t)(sp - start);
            }
            sm.ent[warp][e] = ent;
          }
          __syncwarp();
          if (lane < wdt) pool[poff + lane] = packed_word(lane, wdt, 64, [&](uint64_t e) { return sm.ent[warp][e]; });
          __syncwarp();
        } else {
          const uint64_t plo = st[si] >> 9;
          const uint64_t phi = ((si + 1 < nsb) ? en[si] : last - 1) >> 9;
          for (uint64_t q = lane; q < 64ull * wdt; q += 32)
            pool[poff + q] = packed_word(q, wdt, 4096, [&](uint64_t e) -> uint64_t {
              const uint64_t k = 4096 * si + e;
              return k < m ? batch_select_by_rank(t_b, bits, rank, W, tailmask, plo, phi, k, a.err) : 0;
            });
        }
      }
      __syncthreads();
    }
    // m_superblock
    uint64_t* __restrict__ sbw = a.sbw[t_b] + a.sbo[t];
    const uint64_t sb_nwords = (nsb * logn + 63) / 64;
    for (uint64_t q = tid; q < sb_nwords; q += THREADS)
      sbw[q] = packed_word(q, logn, nsb, [&](uint64_t i) { return st[i]; });
    __syncthreads();
    if (tid == 0) {
      info[4 + (1 - t_b)] = sm.run;
      info[6 + (1 - t_b)] = sm.nlong;
    }
    __syncthreads();
  }
}

template <int THREADS, int IPT>
__global__ void __launch_bounds__(THREADS, 2048 / THREADS / 2) batch_build_kernel(BatchArgs a) {
  __shared__ BatchSmem<THREADS> sm;
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  uint32_t phases = 0;  // bit b: parity of staging buffer b's next completion
  for (;;) {
    if (threadIdx.x == 0) sm.item = atomicAdd(a.queue, 1u);
    __syncthreads();
    const uint32_t item = sm.item;
    __syncthreads();
    if (item >= a.T) break;
    batch_text<THREADS, IPT>(a, a.order[item], sm, phases);
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host

struct BatchVariant {
  int threads, ipt;
  void (*kernel)(BatchArgs);
};

static const BatchVariant kBatchVariants[] = {
    {256, 4, batch_build_kernel<256, 4>},   {256, 8, batch_build_kernel<256, 8>},
    {256, 16, batch_build_kernel<256, 16>}, {512, 4, batch_build_kernel<512, 4>},
    {512, 8, batch_build_kernel<512, 8>},   {512, 16, batch_build_kernel<512, 16>},
    {1024, 4, batch_build_kernel<1024, 4>}, {1024, 8, batch_build_kernel<1024, 8>},
};
constexpr int kNumBatchVariants = sizeof(kBatchVariants) / sizeof(kBatchVariants[0]);

struct BatchImpl {
  uint64_t T = 0;
  int L = 0;
  uint32_t flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<uint64_t> n, so, bo, ro, sao, mo, deo, sbo, poo[2];
  uint64_t bits_words = 0, rank_words = 0, samp_words = 0, mark_words = 0, desc_words = 0, sbw_words = 0;
  DevBuf in, d_so, d_order, d_bo, d_ro, d_sao, d_mo, d_deo, d_sbo, d_poo[2];
  DevBuf bits, rank, samples, marks, desc[2], sbw[2], pool[2], info, queue, err;
  std::vector<uint64_t> h_info;
  int variant = -1;
  float tune_ms[kNumBatchVariants] = {0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool info_valid = false;
};

static uint64_t logn_host(uint64_t size) {
  const uint64_t cap = (size + 63) / 64 * 64;
  return hi64(cap) + 1;
}

// Pool words one text may need for one polarity: every superblock mini at
// most logn words, plus for the long superblocks (disjoint spans longer than
// logn^4, so fewer than size / logn^4 of them) 64 * logn words each.
static uint64_t pool_bound(uint64_t size) {
  const uint64_t logn = logn_host(size);
  const uint64_t logn4 = (uint64_t)(uint32_t)(logn * logn * logn * logn);
  const uint64_t nsb = size / 4096 + 2;
  return nsb * logn + (logn4 ? size / logn4 : 0) * 64 * logn + 1;
}

static BatchArgs batch_args(BatchImpl& b) {
  BatchArgs a;
  a.sym = b.in.as<uint8_t>();
  a.so = b.d_so.as<uint64_t>();
  a.order = b.d_order.as<uint32_t>();
  a.T = b.T;
  a.L = b.L;
  a.flags = b.flags;
  a.bits = b.bits.as<uint64_t>();
  a.bo = b.d_bo.as<uint64_t>();
  a.rank = b.rank.as<uint64_t>();
  a.ro = b.d_ro.as<uint64_t>();
  a.samples = b.samples.as<uint32_t>();
  a.sao = b.d_sao.as<uint64_t>();
  a.marks = b.marks.as<uint64_t>();
  a.mo = b.d_mo.as<uint64_t>();
  a.deo = b.d_deo.as<uint64_t>();
  a.sbo = b.d_sbo.as<uint64_t>();
  for (int t = 0; t < 2; ++t) {
    a.desc[t] = b.desc[t].as<uint64_t>();
    a.sbw[t] = b.sbw[t].as<uint64_t>();
    a.pool[t] = b.pool[t].as<uint64_t>();
    a.poo[t] = b.d_poo[t].as<uint64_t>();
  }
  a.info = b.info.as<uint64_t>();
  a.queue = b.queue.as<uint32_t>();
  a.err = b.err.as<uint32_t>();
  return a;
}

static int batch_grid(const BatchVariant& v, uint64_t T) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.kernel, v.threads, 0);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t g = (uint64_t)std::max(1, per_sm) * (uint64_t)std::max(1, sms);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, T));
}

// the whole build: clear the bits and the queue, run the persistent kernel
static int batch_enqueue(BatchImpl& b, int variant) {
  cudaStream_t s = b.stream;
  const BatchVariant& v = kBatchVariants[variant];
  WTG_CK(cudaMemsetAsync(b.bits.p, 0, b.bits_words * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(b.queue.p, 0, sizeof(uint32_t), s));
  count_launch();
  v.kernel<<<batch_grid(v, b.T), v.threads, 0, s>>>(batch_args(b));
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

BatchImpl* batch_new() { return new (std::nothrow) BatchImpl(); }

void batch_delete(BatchImpl* b) {
  if (!b) return;
  cudaStream_t s = b->stream;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  DevBuf* bufs[] = {&b->in,   &b->d_so,   &b->d_order, &b->d_bo,   &b->d_ro,      &b->d_sao,     &b->d_mo,
                    &b->d_deo, &b->d_sbo, &b->d_poo[0], &b->d_poo[1], &b->bits,   &b->rank,      &b->samples,
                    &b->marks, &b->desc[0], &b->desc[1], &b->sbw[0],  &b->sbw[1], &b->pool[0],   &b->pool[1],
                    &b->info,  &b->queue, &b->err};
  for (DevBuf* d : bufs) d->release(s);
  cudaStreamSynchronize(s);
  if (b->own_stream) cudaStreamDestroy(s);
  delete b;
}

int batch_plan(BatchImpl& b, const uint64_t* lengths, uint64_t T, int L, uint32_t flags, cudaStream_t s,
               bool own_stream) {
  int rc;
  if (T == 0 || T >= (1ull << 31)) return fail(WTG_ERR_INVALID, "ntexts must be 1 .. 2^31 - 1");
  if (L < 1 || L > BATCH_LMAX) return fail(WTG_ERR_INVALID, "batched builds take 1..4 levels");
  if (flags & ~WTG_ALL) return fail(WTG_ERR_INVALID, "unknown flags");
  if (flags & (WTG_SELECT1 | WTG_SELECT0)) flags |= WTG_RANK;  // the long blocks search the rank table
  b.T = T;
  b.L = L;
  b.flags = flags;
  b.stream = s;
  b.own_stream = own_stream;
  b.n.assign(lengths, lengths + T);
  b.so.assign(T + 1, 0);
  b.bo.assign(T + 1, 0);
  b.ro.assign(T + 1, 0);
  b.sao.assign(T + 1, 0);
  b.mo.assign(T + 1, 0);
  b.deo.assign(T + 1, 0);
  b.sbo.assign(T + 1, 0);
  b.poo[0].assign(T + 1, 0);
  b.poo[1].assign(T + 1, 0);
  for (uint64_t t = 0; t < T; ++t) {
    const uint64_t n = b.n[t];
    if (n >= (1ull << 31) / (uint64_t)L) return fail(WTG_ERR_INVALID, "a text's bits must stay below 2^31");
    const uint64_t size = (uint64_t)L * n;
    const uint64_t W = (size + 63) / 64;
    const uint64_t nsbc = size / 4096 + 2;
    const uint64_t logn = logn_host(size);
    b.so[t + 1] = b.so[t] + n;
    b.bo[t + 1] = b.bo[t] + (W + 16 + 15) / 16 * 16;  // padded to whole 128-byte lines
    b.ro[t + 1] = b.ro[t] + ((W >> 3) + 1) * 2;
    b.sao[t + 1] = b.sao[t] + W + 2;
    b.mo[t + 1] = b.mo[t] + 4 * nsbc;
    b.deo[t + 1] = b.deo[t] + nsbc;
    b.sbo[t + 1] = b.sbo[t] + (nsbc * logn + 63) / 64 + 1;
    const uint64_t pb = pool_bound(size);
    b.poo[0][t + 1] = b.poo[0][t] + pb;
    b.poo[1][t + 1] = b.poo[1][t] + pb;
  }
  b.bits_words = b.bo[T];
  b.rank_words = b.ro[T];
  std::vector<uint32_t> order(T);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return b.n[x] > b.n[y]; });

  auto up = [&](DevBuf& d, const void* h, size_t bytes) -> int {
    int r;
    if ((r = d.ensure(std::max<size_t>(bytes, 8), s))) return r;
    WTG_CK(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, s));
    return WTG_OK;
  };
  if ((rc = b.in.ensure(b.so[T] + 16, s))) return rc;
  if ((rc = up(b.d_so, b.so.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_order, order.data(), T * 4))) return rc;
  if ((rc = up(b.d_bo, b.bo.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_ro, b.ro.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_sao, b.sao.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_mo, b.mo.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_deo, b.deo.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_sbo, b.sbo.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_poo[0], b.poo[0].data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_poo[1], b.poo[1].data(), (T + 1) * 8))) return rc;
  if ((rc = b.bits.ensure(b.bits_words * 8 + 64, s))) return rc;
  if ((rc = b.rank.ensure(b.rank_words * 8 + 64, s))) return rc;
  if ((rc = b.samples.ensure(b.sao[T] * 4 + 64, s))) return rc;
  if ((rc = b.marks.ensure(b.mo[T] * 8 + 64, s))) return rc;
  for (int t = 0; t < 2; ++t) {
    if ((rc = b.desc[t].ensure(b.deo[T] * 8 + 64, s))) return rc;
    if ((rc = b.sbw[t].ensure(b.sbo[T] * 8 + 64, s))) return rc;
    if ((rc = b.pool[t].ensure(b.poo[t][T] * 8 + 64, s))) return rc;
  }
  if ((rc = b.info.ensure(T * 8 * 8, s))) return rc;
  if ((rc = b.queue.ensure(8, s))) return rc;
  if ((rc = b.err.ensure(8, s))) return rc;
  WTG_CK(cudaMemsetAsync(b.info.p, 0, T * 64, s));
  WTG_CK(cudaMemsetAsync(b.err.p, 0, 8, s));
  WTG_CK(cudaStreamSynchronize(s));  // the host vectors above must outlive the copies
  return WTG_OK;
}

// the build (clear, launch) captured once in a CUDA graph for replay
static int batch_capture(BatchImpl& b) {
  int rc;
  cudaStream_t s = b.stream;
  WTG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  rc = batch_enqueue(b, b.variant);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) return cuda_fail(ce, "capture of the batched build");
  b.graph = g;
  WTG_CK(cudaGraphInstantiate(&b.exec, g, 0));
  return WTG_OK;
}

// Times every launch shape once (after one warm-up run of each) on the
// batch's own input and keeps the fastest; then captures the build in a graph.
static int batch_tune_and_capture(BatchImpl& b) {
  int rc;
  cudaStream_t s = b.stream;
  cudaEvent_t e0, e1;
  WTG_CK(cudaEventCreate(&e0));
  WTG_CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_v = 0;
  for (int v = 0; v < kNumBatchVariants; ++v) {
    if ((rc = batch_enqueue(b, v))) break;
    WTG_CK(cudaEventRecord(e0, s));
    if ((rc = batch_enqueue(b, v))) break;
    WTG_CK(cudaEventRecord(e1, s));
    WTG_CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    b.tune_ms[v] = ms;
    if (ms < best) {
      best = ms;
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  b.variant = best_v;
  return batch_capture(b);
}

int batch_set_shape(BatchImpl& b, int threads, int ipt) {
  for (int v = 0; v < kNumBatchVariants; ++v) {
    if (kBatchVariants[v].threads == threads && kBatchVariants[v].ipt == ipt) {
      if (b.exec) cudaGraphExecDestroy(b.exec);
      if (b.graph) cudaGraphDestroy(b.graph);
      b.exec = nullptr;
      b.graph = nullptr;
      b.variant = v;
      return batch_capture(b);
    }
  }
  return fail(WTG_ERR_INVALID, "no such launch shape (threads 256/512/1024, symbols per thread 4/8/16)");
}

int batch_run(BatchImpl& b) {
  int rc;
  b.info_valid = false;
  if (!b.exec) {
    if ((rc = batch_tune_and_capture(b))) return rc;
  }
  count_launch();
  WTG_CK(cudaGraphLaunch(b.exec, b.stream));
  return WTG_OK;
}

int batch_sync(BatchImpl& b, uint32_t* err_out) {
  WTG_CK(cudaStreamSynchronize(b.stream));
  uint32_t e = 0;
  WTG_CK(cudaMemcpy(&e, b.err.p, sizeof(e), cudaMemcpyDeviceToHost));
  *err_out = e;
  b.h_info.resize(b.T * 8);
  WTG_CK(cudaMemcpy(b.h_info.data(), b.info.p, b.T * 64, cudaMemcpyDeviceToHost));
  b.info_valid = true;
  return WTG_OK;
}

// per-text info and outputs (after batch_sync)
int batch_text_info(const BatchImpl& b, uint64_t t, uint64_t info[8]) {
  if (t >= b.T) return fail(WTG_ERR_RANGE, "text index out of range");
  if (!b.info_valid) return fail(WTG_ERR_INVALID, "sync the batch first");
  const uint64_t size = (uint64_t)b.L * b.n[t];
  info[0] = b.n[t];
  info[1] = b.L;
  info[2] = (size + 63) / 64;
  info[3] = b.ro[t + 1] - b.ro[t];
  info[4] = b.h_info[8 * t + 0];
  info[5] = b.h_info[8 * t + 1];
  info[6] = b.variant >= 0 ? (uint64_t)kBatchVariants[b.variant].threads : 0;
  info[7] = b.variant >= 0 ? (uint64_t)kBatchVariants[b.variant].ipt : 0;
  return WTG_OK;
}

int batch_select_info(const BatchImpl& b, uint64_t t, int t_b, uint64_t info[8]) {
  if (t >= b.T) return fail(WTG_ERR_RANGE, "text index out of range");
  if (!b.info_valid) return fail(WTG_ERR_INVALID, "sync the batch first");
  if (!(b.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select support not built");
  const uint64_t size = (uint64_t)b.L * b.n[t];
  const uint64_t m = b.h_info[8 * t + (t_b ? 0 : 1)];
  const uint64_t logn = logn_host(size);
  const uint64_t nsb = (m + 4095) >> 12;
  info[0] = size;
  info[1] = m;
  info[2] = logn;
  info[3] = (uint64_t)(uint32_t)(logn * logn * logn * logn);
  info[4] = nsb;
  info[5] = b.h_info[8 * t + (t_b ? 6 : 7)] ? 1 : 0;
  info[6] = (nsb * logn + 63) / 64;
  info[7] = b.h_info[8 * t + (t_b ? 4 : 5)];
  return WTG_OK;
}

int batch_get(const BatchImpl& b, uint64_t t, int what, int t_b, void* dst, uint64_t nwords) {
  if (t >= b.T) return fail(WTG_ERR_RANGE, "text index out of range");
  if (!b.info_valid) return fail(WTG_ERR_INVALID, "sync the batch first");
  const uint64_t size = (uint64_t)b.L * b.n[t];
  const uint64_t* src = nullptr;
  uint64_t have = 0;
  if (what == 0) {
    src = b.bits.as<uint64_t>() + b.bo[t];
    have = (size + 63) / 64;
  } else if (what == 1) {
    if (!(b.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "rank support not built");
    src = b.rank.as<uint64_t>() + b.ro[t];
    have = b.ro[t + 1] - b.ro[t];
  } else {
    uint64_t si[8];
    int rc;
    if ((rc = batch_select_info(b, t, t_b, si))) return rc;
    if (what == 2) {
      src = b.sbw[t_b].as<uint64_t>() + b.sbo[t];
      have = si[6];
    } else if (what == 3) {
      src = b.desc[t_b].as<uint64_t>() + b.deo[t];
      have = si[4];
    } else {
      src = b.pool[t_b].as<uint64_t>() + b.poo[t_b][t];
      have = si[7];
    }
  }
  if (nwords != have) return fail(WTG_ERR_INVALID, "nwords must equal the output's size");
  if (nwords) {
    WTG_CK(cudaMemcpyAsync(dst, src, nwords * 8, cudaMemcpyDeviceToHost, b.stream));
    WTG_CK(cudaStreamSynchronize(b.stream));
  }
  return WTG_OK;
}

void* batch_input(BatchImpl& b) { return b.in.p; }
cudaStream_t batch_stream(const BatchImpl& b) { return b.stream; }
uint64_t batch_total_symbols(const BatchImpl& b) { return b.so[b.T]; }

int batch_tuning(const BatchImpl& b, int* threads, int* ipt, float* ms, int nms) {
  if (b.variant < 0) return fail(WTG_ERR_INVALID, "the batch has not run yet");
  *threads = kBatchVariants[b.variant].threads;
  *ipt = kBatchVariants[b.variant].ipt;
  for (int v = 0; v < nms && v < kNumBatchVariants; ++v) ms[v] = b.tune_ms[v];
  return WTG_OK;
}

}  // namespace wtg
