// wtg_batch.cu -- batched builds: many independent texts, each with its own
// wavelet tree (level bitvector of L <= 4 levels), rank_support_v<1> and
// select_support_mcl<1>/<0>, all in one persistent launch.
//
// The reference builds one sequence per WT() call (levelWT/WT.C:43-227,
// driven by levelWT/WTTime.C:78-103); a batch there is a loop of calls.  Here
// one persistent kernel pulls work items from a device queue.  The item list
// is made at plan time, in phase order, each phase's items by decreasing text
// length:
//   H (text, tile)        the key histogram of one tile of the text;
//                         the text's last H item to finish turns the tiles'
//                         histograms into per-tile prefixes and totals
//   W (text, level, tile) the tile's bits of one level.  Level l of a text is
//                         the text stably sorted by the top l bits
//                         (levelWT/WT.C:118-190), so the symbols of (level l,
//                         key k) form one contiguous bit run starting at
//                         l*n + (symbols whose key is below k), and a tile's
//                         piece of it starts after the earlier tiles' members
//                         (the H prefixes): every tile and level is written
//                         from the text directly, no level-by-level passes
//   R (text, rank tile)   rank_support_v entries and select sample marks of
//                         256 superblocks, the ones before the tile from a
//                         decoupled look-back over the text's rank tiles
//                         (the reference layout and final-superblock rule)
//   S (text)              select_support_mcl per polarity: long/mini choice,
//                         widths, pool offsets (block scan), mini blocks from
//                         the samples, long blocks by rank-table search,
//                         m_superblock packing.
// An item first waits (bounded) until its text's previous phase is complete:
// per-text counters, bumped after each item's writes are fenced.  Every item
// waits only on items taken from the queue before it, by CTAs that are
// running, so the launch always completes.  Data another CTA wrote is read
// through L2 (ld.cg, or bulk copies).
// Every output has the layout of the single-sequence build.  The pool region
// of each text is sized by a bound that holds for any input (see plan), so
// the layout is fixed by the text lengths alone.  The launch shape (symbols
// per thread per chunk, chunks per W tile) is picked by timing the candidates
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
constexpr int BATCH_BINS = 1 << BATCH_LMAX;
constexpr uint32_t BATCH_INVALID = 0xFFFFFFFFu;
constexpr int BT = 256;                       // threads per CTA
constexpr int BNW = BT / 32;                  // warps per CTA
constexpr int BATCH_MAX_CHUNK = BT * 16;      // symbols per chunk of the widest launch shape
constexpr int RT_ITER = 8;                    // rows of BT words per rank tile
constexpr int RT_SB = RT_ITER * BT / 8;       // superblocks per rank tile (R item)

// work item: x = text, y = kind | level << 8, z = tile
enum : uint32_t { IT_H = 0, IT_W = 1, IT_R = 2, IT_S = 3 };
// per-text completion counters: done[4 t + DN_*]
enum : uint32_t { DN_H = 0, DN_HREADY = 1, DN_W = 2, DN_R = 3 };

struct BatchArgs {
  const uint8_t* sym;     // concatenated texts
  const uint64_t* so;     // symbol offset of each text, T + 1
  uint64_t T;
  int L;
  uint32_t flags;
  uint64_t tile;          // symbols per H / W tile
  const uint4* items;
  uint32_t nitems;
  const uint64_t* hb;     // first H tile of each text, T + 1
  uint32_t* thist;        // per H tile: BATCH_BINS counts, made exclusive prefixes by the text's last H item
  uint32_t* ttot;         // per text: BATCH_BINS totals
  const uint64_t* rb;     // first rank tile of each text, T + 1
  uint64_t* rstat;        // look-back status per rank tile
  uint32_t* done;         // 4 counters per text
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

struct BatchSmem {
  uint4 item[2];  // the item being processed and the next one (taken early)
  uint32_t hist[BATCH_BINS];
  uint32_t part[16][BATCH_BINS];
  uint64_t base[BATCH_SLOTS];
  uint64_t carry[BATCH_SLOTS];
  uint32_t cnt[BNW][BATCH_SLOTS];
  uint64_t start[BNW][BATCH_SLOTS];
  uint64_t wsum[BNW];
  uint64_t run;
  uint32_t nlong;
  uint32_t flag;
  uint32_t sb[RT_SB];
  uint64_t prefix;
  uint64_t ent[BNW][64];
  // W: two staging buffers for chunks of up to BATCH_MAX_CHUNK symbols (plus
  // the text's offset from a 16-byte boundary), filled by cp.async.bulk
  alignas(16) uint8_t stage[2][BATCH_MAX_CHUNK + 32];
  alignas(8) uint64_t bar[2];
};

__device__ __forceinline__ uint64_t batch_logn(uint64_t size) {
  const uint64_t cap = (size + 63) / 64 * 64;
  return hi64(cap) + 1;
}

// Waits until *ctr reaches `need` (thread 0 spins, bounded; on expiry the
// error is recorded and the item goes on with whatever is there), then the
// whole CTA proceeds and sees the writes fenced before the counter bumps.
__device__ __forceinline__ void batch_wait(const uint32_t* ctr, uint32_t need, uint32_t* err) {
  if (threadIdx.x == 0) {
    uint32_t spins = 0, ns = 32;
    const uint32_t limit = c_wait_limit[0];
    while (*((volatile const uint32_t*)ctr) < need) {
      if (++spins > limit) {
        atomicCAS(err, 0u, (uint32_t)DERR_LOOKBACK_TIMEOUT);
        break;
      }
      __nanosleep(ns);
      if (ns < 1024) ns <<= 1;
    }
    __threadfence();
  }
  __syncthreads();
}

// After the CTA's writes (every thread fences its own): bumps *ctr; returns
// the previous count to thread 0
__device__ __forceinline__ uint32_t batch_signal(uint32_t* ctr) {
  __threadfence();
  __syncthreads();
  uint32_t prev = 0;
  if (threadIdx.x == 0) {
    __threadfence();
    prev = atomicAdd(ctr, 1u);
  }
  return prev;
}

// block-wide exclusive scan of one u64 per thread; returns the prefix and
// the block total through *total
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, BatchSmem& sm, uint64_t* total) {
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
  for (int w = 0; w < BNW; ++w) {
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
// (both written by other CTAs: read through L2)
__device__ __forceinline__ uint64_t batch_select_by_rank(int t_b, const uint64_t* __restrict__ words,
                                                         const uint64_t* __restrict__ rank, uint64_t W,
                                                         uint64_t tailmask, uint64_t lo, uint64_t hi, uint64_t k,
                                                         uint32_t* err) {
  const uint64_t last_sb = W >> 3;  // superblock entries 0 .. W/8
  if (hi > last_sb) hi = last_sb;
  if (lo > hi) lo = hi;
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) >> 1;
    const uint64_t r = __ldcg(rank + 2 * mid);
    if ((t_b ? r : 512 * mid - r) <= k) lo = mid;
    else hi = mid - 1;
  }
  const uint64_t r = __ldcg(rank + 2 * lo);
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

// ---- H item: the key histogram of symbols [c0, c1) of a text.  The order of
// the symbols does not matter here, so each thread reads 16 at a time and
// counts the low-L-bit values of a 32-bit word bit-sliced (L <= 2) or
// bytewise (L = 3, 4); bin 0 is what remains.
__device__ void batch_h_item(const BatchArgs& a, uint32_t t, uint32_t j, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const int L = a.L;
  const uint32_t nbin = 1u << L, vmask = nbin - 1;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint64_t c0 = (uint64_t)j * a.tile, c1 = min(n, c0 + a.tile), cnt = c1 - c0;
  const uint8_t* __restrict__ in = a.sym + a.so[t] + c0;
  if (tid < BATCH_BINS) sm.hist[tid] = 0;
  __syncthreads();
  {
    uint32_t c[BATCH_BINS];
#pragma unroll
    for (int b = 0; b < BATCH_BINS; ++b) c[b] = 0;
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
        for (int b = 1; b < BATCH_BINS; ++b)
          if ((uint32_t)b < nbin) c[b] += __popc(__vcmpeq4(x, (uint32_t)b * 0x01010101u)) >> 3;
      }
    };
    const uint64_t head = min(cnt, (uint64_t)((16u - ((uintptr_t)in & 15u)) & 15u));  // bytes before a 16-byte boundary
    const uint64_t nvec = (cnt - head) / 16;
    const uint64_t rest = head + nvec * 16;
    if (tid < head) count_word(in[tid]);
    if (tid < cnt - rest) count_word(in[rest + tid]);
    const uint4* vin = reinterpret_cast<const uint4*>(in + head);
    uint64_t q = tid;
    for (; q + BT < nvec; q += 2 * BT) {
      const uint4 u = __ldg(vin + q), v = __ldg(vin + q + BT);
      count_word(u.x); count_word(u.y); count_word(u.z); count_word(u.w);
      count_word(v.x); count_word(v.y); count_word(v.z); count_word(v.w);
    }
    if (q < nvec) {
      const uint4 u = __ldg(vin + q);
      count_word(u.x); count_word(u.y); count_word(u.z); count_word(u.w);
    }
#pragma unroll
    for (int b = 1; b < BATCH_BINS; ++b) {
      if ((uint32_t)b >= nbin) continue;
      const uint32_t s = __reduce_add_sync(0xffffffffu, c[b]);
      if (lane == 0 && s) atomicAdd(&sm.hist[b], s);
    }
  }
  __syncthreads();
  uint32_t* __restrict__ th = a.thist + (a.hb[t] + j) * BATCH_BINS;
  if (tid < BATCH_BINS) {
    uint32_t v = 0;
    if (tid == 0) {
      uint32_t others = 0;
      for (uint32_t b = 1; b < nbin; ++b) others += sm.hist[b];
      v = (uint32_t)cnt - others;
    } else if (tid < nbin) {
      v = sm.hist[tid];
    }
    th[tid] = v;
  }
  const uint32_t prev = batch_signal(&a.done[4 * t + DN_H]);
  if (tid == 0) sm.flag = prev;
  __syncthreads();
  const uint32_t J = (uint32_t)(a.hb[t + 1] - a.hb[t]);
  if (sm.flag + 1 != J) return;
  // the text's last H item: per-tile exclusive prefixes (in place) and
  // totals; thread (part, bin) handles tiles part, part + 16, ...
  if (tid == 0) __threadfence();
  __syncthreads();
  uint32_t* __restrict__ h0 = a.thist + a.hb[t] * BATCH_BINS;
  const uint32_t b = tid & (BATCH_BINS - 1), part = tid >> 4;
  const uint32_t per = (J + 15) / 16, j0 = part * per, j1 = min(J, j0 + per);
  uint32_t s = 0;
  for (uint32_t q = j0; q < j1; ++q) s += __ldcg(h0 + q * BATCH_BINS + b);
  sm.part[part][b] = s;
  __syncthreads();
  uint32_t before = 0, total = 0;
  for (uint32_t p = 0; p < 16; ++p) {
    before += p < part ? sm.part[p][b] : 0u;
    total += sm.part[p][b];
  }
  for (uint32_t q = j0; q < j1; ++q) {
    const uint32_t c = __ldcg(h0 + q * BATCH_BINS + b);
    h0[q * BATCH_BINS + b] = before;
    before += c;
  }
  if (part == 0) a.ttot[(uint64_t)t * BATCH_BINS + b] = total;
  batch_signal(&a.done[4 * t + DN_HREADY]);
}

// ---- W item: the bits of level l for symbols [c0, c1) of a text.  Level 0
// holds every symbol in order: a warp's row pair is one 64-bit word.  Level
// l >= 1 has 2^l runs (keys); per chunk of BT * IPT symbols a warp counts
// its rows' members of each run (one ballot per bit plane and row; run masks
// from logic ops), the block places the warps' pieces after the run's carry,
// and each warp appends its pieces, compacting the level's plane to the run
// with one OR-reduction of 1 << rank per row.  Words a piece shares with a
// neighbouring piece (its first and last) are ORed with 64-bit atomics;
// words inside it are stored.
template <int IPT, int LL>
__device__ void batch_w_item(const BatchArgs& a, uint32_t t, int l, uint32_t j, BatchSmem& sm, uint32_t& phases) {
  constexpr uint64_t CH = (uint64_t)BT * IPT;
  static_assert(CH <= BATCH_MAX_CHUNK, "chunk larger than the staging buffers");
  static_assert(IPT % 2 == 0, "level 0 rows are stored in pairs");
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t vmask = (1u << LL) - 1, lt = (1u << lane) - 1;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint8_t* __restrict__ in = a.sym + a.so[t];
  uint64_t* __restrict__ bits = a.bits + a.bo[t];
  const uint64_t cb = (uint64_t)j * a.tile, ce = min(n, cb + a.tile);
  const int bs = LL - 1 - l;      // the bit plane of level l
  const int q0 = (1 << l) - 1;    // first slot of level l
  const int nk = 1 << l;          // its runs
  // run starts: l * n + symbols of keys below k; the tile's piece after the earlier tiles' members
  if (tid < (uint32_t)nk) {
    const uint32_t* tot = a.ttot + (uint64_t)t * BATCH_BINS;
    const uint32_t* pre = a.thist + (a.hb[t] + j) * BATCH_BINS;
    uint64_t below = 0, mine = 0;
    for (uint32_t b = 0; b < (1u << LL); ++b) {
      const uint32_t key = b >> (LL - l);
      if (key < tid) below += __ldcg(tot + b);
      if (key == tid) mine += __ldcg(pre + b);
    }
    sm.base[q0 + tid] = (uint64_t)l * n + below;
    sm.carry[q0 + tid] = mine;
  }
  // chunks are staged by thread 0 one ahead: from the 16-byte boundary at
  // or below the chunk (the input has 16 bytes of padding after the last
  // text, so the rounded-up tail stays inside it); tile starts are multiples
  // of 16, so every chunk has the same offset from its boundary
  const uint32_t off = (uint32_t)((uintptr_t)in & 15u);
  auto stage_chunk = [&](uint64_t c, int buf) {
    const uint64_t cnt = min(CH, ce - c);
    const uint32_t bytes = (uint32_t)((off + cnt + 15) & ~15ull);
    fence_proxy_async_smem();
    mbar_expect_tx(&sm.bar[buf], bytes);
    bulk_g2s(sm.stage[buf], in + c - off, bytes, &sm.bar[buf]);
  };
  __syncthreads();
  int cur = 0;
  if (tid == 0 && ce > cb) stage_chunk(cb, 0);
  for (uint64_t c0 = cb; c0 < ce; c0 += CH, cur ^= 1) {
    if (tid == 0 && c0 + CH < ce) stage_chunk(c0 + CH, cur ^ 1);  // its last readers passed the previous barrier
    mbar_wait(&sm.bar[cur], (phases >> cur) & 1u, a.err);
    phases ^= 1u << cur;
    const uint8_t* const st = sm.stage[cur] + off;
    const uint64_t s0 = c0 + (uint64_t)warp * 32 * IPT;
    uint32_t v[IPT];
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const uint64_t i = s0 + 32 * r + lane;
      v[r] = i < ce ? (st[i - c0] & vmask) : BATCH_INVALID;
    }
    if (l == 0) {
      // level 0: bit bs of every symbol, in order; rows 2h and 2h + 1 form
      // the 64-bit word (s0 + 64 h) / 64 of the text's bits
#pragma unroll
      for (int h = 0; h < IPT / 2; ++h) {
        const bool va = v[2 * h] != BATCH_INVALID, vb = v[2 * h + 1] != BATCH_INVALID;
        const uint32_t lo = __ballot_sync(0xffffffffu, va && ((v[2 * h] >> bs) & 1u));
        const uint32_t hi = __ballot_sync(0xffffffffu, vb && ((v[2 * h + 1] >> bs) & 1u));
        const uint64_t first = s0 + 64 * h;
        if (lane == 0 && first < ce) {
          const uint64_t wv = ((uint64_t)hi << 32) | lo;
          // the text's last level-0 word may share bits with level 1
          if (first + 64 <= n) bits[first >> 6] = wv;
          else if (wv) atomicOr((unsigned long long*)&bits[first >> 6], (unsigned long long)wv);
        }
      }
      __syncthreads();  // the staging buffer is refilled after every warp has read it
      continue;
    }
    constexpr int NKMAX = 1 << (LL - 1);  // keys of the deepest level
    uint32_t cnt[NKMAX];
#pragma unroll
    for (int k = 0; k < NKMAX; ++k) cnt[k] = 0;
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const bool valid = v[r] != BATCH_INVALID;
      uint32_t P[LL];
#pragma unroll
      for (int jj = 0; jj < LL; ++jj) P[jj] = __ballot_sync(0xffffffffu, valid && ((v[r] >> jj) & 1u));
      const uint32_t V = __ballot_sync(0xffffffffu, valid);
#pragma unroll
      for (int k = 0; k < NKMAX; ++k)
        if (k < nk) cnt[k] += __popc(batch_run_mask<LL>(P, V, l, (uint32_t)k));
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NKMAX; ++k)
        if (k < nk) sm.cnt[warp][q0 + k] = cnt[k];
    }
    __syncthreads();
    if (tid < (uint32_t)nk) {
      const int q = q0 + tid;
      uint64_t run = sm.carry[q];
      for (int w = 0; w < BNW; ++w) {
        sm.start[w][q] = run;
        run += sm.cnt[w][q];
      }
      sm.carry[q] = run;
    }
    __syncthreads();
    uint64_t acc[NKMAX], word[NKMAX];
    uint32_t fill[NKMAX];
    bool shared_word[NKMAX];
#pragma unroll
    for (int k = 0; k < NKMAX; ++k) {
      const uint64_t dest = k < nk ? sm.base[q0 + k] + sm.start[warp][q0 + k] : 0;
      word[k] = dest >> 6;
      fill[k] = (uint32_t)(dest & 63);
      shared_word[k] = fill[k] != 0;  // the first word may hold the previous piece's tail
      acc[k] = 0;
    }
#pragma unroll
    for (int r = 0; r < IPT; ++r) {
      const bool valid = v[r] != BATCH_INVALID;
      uint32_t P[LL];
#pragma unroll
      for (int jj = 0; jj < LL; ++jj) P[jj] = __ballot_sync(0xffffffffu, valid && ((v[r] >> jj) & 1u));
      const uint32_t V = __ballot_sync(0xffffffffu, valid);
      uint32_t plane = P[0];
#pragma unroll
      for (int jj = 1; jj < LL; ++jj) plane = jj == bs ? P[jj] : plane;
#pragma unroll
      for (int k = 0; k < NKMAX; ++k) {
        if (k >= nk) continue;
        const uint32_t m = batch_run_mask<LL>(P, V, l, (uint32_t)k);
        const uint32_t cm = __popc(m);
        if (cm == 0) continue;
        const uint32_t one = ((m & plane) >> lane) & 1u ? (1u << __popc(m & lt)) : 0u;
        const uint32_t comp = __reduce_or_sync(0xffffffffu, one);
        acc[k] |= (uint64_t)comp << fill[k];
        if (fill[k] + cm >= 64) {
          if (lane == 0 && acc[k]) {
            if (shared_word[k]) atomicOr((unsigned long long*)&bits[word[k]], (unsigned long long)acc[k]);
            else bits[word[k]] = acc[k];
          }
          acc[k] = fill[k] ? ((uint64_t)comp >> (64 - fill[k])) : 0;
          fill[k] = fill[k] + cm - 64;
          ++word[k];
          shared_word[k] = false;
        } else {
          fill[k] += cm;
        }
      }
    }
    // the piece's last (partial) word is shared with the next piece
#pragma unroll
    for (int k = 0; k < NKMAX; ++k)
      if (k < nk && lane == 0 && fill[k] && acc[k])
        atomicOr((unsigned long long*)&bits[word[k]], (unsigned long long)acc[k]);
    __syncthreads();
  }
  batch_signal(&a.done[4 * t + DN_W]);
}

// ---- R item: rank_support_v entries and select marks of rank tile r (RT_SB
// superblocks) of a text's bitvector; the ones before the tile from a
// decoupled look-back over the text's rank tiles (taken from the queue in
// order, so every predecessor has started).  The tile holding the final
// superblock writes the arg counts; last args go to the text's info.
__device__ void batch_r_item(const BatchArgs& a, uint32_t t, uint32_t r, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g8 = lane & 7;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint64_t size = (uint64_t)a.L * n;
  const uint64_t W = (size + 63) / 64, NB = W >> 3;
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  const uint32_t flags = a.flags;
  const bool sel1 = flags & WTG_SELECT1, sel0 = flags & WTG_SELECT0;
  const uint64_t* __restrict__ words = a.bits + a.bo[t];
  uint64_t* __restrict__ rank = a.rank + a.ro[t];
  uint32_t* __restrict__ samples = a.samples + a.sao[t];
  const uint64_t samp_last = W + 1;
  const uint64_t nsbc = size / 4096 + 2;
  uint64_t* __restrict__ starts1 = a.marks + a.mo[t];
  uint64_t* __restrict__ starts0 = starts1 + nsbc;
  uint64_t* __restrict__ ends1 = starts0 + nsbc;
  uint64_t* __restrict__ ends0 = ends1 + nsbc;
  uint64_t* __restrict__ info = a.info + 8 * (uint64_t)t;
  uint64_t* __restrict__ status = a.rstat + a.rb[t];
  const uint64_t wbase = (uint64_t)r * (RT_ITER * BT);
  uint64_t w[RT_ITER];
  uint32_t c[RT_ITER], inc[RT_ITER];
#pragma unroll
  for (int i = 0; i < RT_ITER; ++i) {
    const uint64_t wi = wbase + i * BT + tid;
    uint64_t x = wi < W ? __ldcg(words + wi) : 0ull;  // written by the W items of other CTAs
    if (wi == W - 1) x &= tailmask;
    w[i] = x;
    c[i] = __popcll(x);
    uint32_t v = c[i];
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {  // inclusive scan within the superblock's 8 lanes
      const uint32_t q = __shfl_up_sync(0xffffffffu, v, o);
      if (g8 >= (uint32_t)o) v += q;
    }
    inc[i] = v;
    if (g8 == 7) sm.sb[i * (BT / 8) + warp * 4 + (lane >> 3)] = v;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int PER = RT_SB / 32;
    uint32_t loc[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      loc[q] = sm.sb[lane * PER + q];
      sum += loc[q];
    }
    uint32_t incw = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t q = __shfl_up_sync(0xffffffffu, incw, o);
      if (lane >= (uint32_t)o) incw += q;
    }
    uint32_t run = incw - sum;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      sm.sb[lane * PER + q] = run;
      run += loc[q];
    }
    const uint64_t total = __shfl_sync(0xffffffffu, incw, 31);
    uint64_t prefix = 0;
    if (r == 0) {
      if (lane == 0) lb_publish(status, r, LB_FLAG_INC, total);
    } else {
      if (lane == 0) lb_publish(status, r, LB_FLAG_AGG, total);
      prefix = lb_lookback_warp(status, r, a.err);
      if (lane == 0) lb_publish(status, r, LB_FLAG_INC, prefix + total);
    }
    if (lane == 0) sm.prefix = prefix;
  }
  __syncthreads();
  const uint64_t tprefix = sm.prefix;
  const uint64_t r_last = W - 8 * NB;  // words of the final superblock
  uint64_t last1 = 0, last0 = 0;
#pragma unroll
  for (int i = 0; i < RT_ITER; ++i) {
    const uint32_t sbl = i * (BT / 8) + warp * 4 + (lane >> 3);
    const uint64_t b = (uint64_t)r * RT_SB + sbl;  // superblock
    const uint64_t wi = wbase + i * BT + tid;
    const uint64_t sb_before = tprefix + sm.sb[sbl];
    const uint32_t excl = inc[i] - c[i];
    const uint32_t sbt = __shfl_sync(0xffffffffu, inc[i], (lane & ~7u) + 7);
    if (flags & WTG_RANK) {
      // field k (1..7) = count before block k; the final superblock writes
      // only fields 1..max(r,1), r = its words (rank_support_v_par.hpp:99-108)
      const uint32_t kmax = (b < NB) ? 7u : (r_last > 1 ? (uint32_t)r_last : 1u);
      uint64_t part = (g8 >= 1 && g8 <= kmax) ? ((uint64_t)excl << (63 - 9 * g8)) : 0ull;
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) part |= __shfl_xor_sync(0xffffffffu, part, o);
      if (g8 == 0 && b <= NB) {
        rank[2 * b] = sb_before;
        rank[2 * b + 1] = part;
      }
    }
    if (b == NB && g8 == 0) {
      info[0] = sb_before + sbt;
      info[1] = size - (sb_before + sbt);
    }
    if (wi < W)
      word_marks(w[i], c[i], sb_before + excl, wi, wi == W - 1 ? tailmask : ~0ull, sel1, sel0, samples, samp_last,
                 starts1, starts0, ends1, ends0, last1, last0);
  }
  const uint64_t e1 = last_arg_end(words, last1, W, tailmask, 1);
  const uint64_t e0 = last_arg_end(words, last0, W, tailmask, 0);
  if (e1) atomicMax((unsigned long long*)&info[2], (unsigned long long)e1);
  if (e0) atomicMax((unsigned long long*)&info[3], (unsigned long long)e0);
  batch_signal(&a.done[4 * t + DN_R]);
}

// ---- S item: select_support_mcl of each polarity of one text
__device__ void batch_s_item(const BatchArgs& a, uint32_t t, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint64_t size = (uint64_t)a.L * n;
  const uint64_t W = (size + 63) / 64;
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  const bool sel1 = a.flags & WTG_SELECT1, sel0 = a.flags & WTG_SELECT0;
  const uint64_t* __restrict__ bits = a.bits + a.bo[t];
  const uint64_t* __restrict__ rank = a.rank + a.ro[t];
  const uint32_t* __restrict__ samples = a.samples + a.sao[t];
  const uint64_t samp_last = W + 1;
  const uint64_t nsbc = size / 4096 + 2;
  const uint64_t* __restrict__ starts1 = a.marks + a.mo[t];
  const uint64_t* __restrict__ starts0 = starts1 + nsbc;
  const uint64_t* __restrict__ ends1 = starts0 + nsbc;
  const uint64_t* __restrict__ ends0 = ends1 + nsbc;
  uint64_t* info = a.info + 8 * (uint64_t)t;
  const uint64_t m1 = __ldcg(info + 0), m0 = __ldcg(info + 1);
  const uint64_t last1 = __ldcg(info + 2), last0 = __ldcg(info + 3);
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
    for (uint64_t i0 = 0; i0 < nsb; i0 += BT) {
      const uint64_t i = i0 + tid;
      uint64_t sz = 0, d = 0;
      if (i < nsb) {
        const uint64_t start = __ldcg(st + i);
        const uint64_t end = (i + 1 < nsb) ? __ldcg(en + i) : last - 1;
        const uint64_t span = end - start;
        const uint64_t lng = span > logn4;
        const uint64_t wdt = lng ? hi64(end) + 1 : hi64(span) + 1;
        d = (lng << 7) | wdt;
        sz = lng ? 64 * wdt : wdt;
        if (lng) atomicAdd(&sm.nlong, 1u);
      }
      uint64_t total;
      const uint64_t off = sm.run + block_excl_scan(sz, sm, &total);
      if (i < nsb) {
        if (off + sz > pool_cap) atomicCAS(a.err, 0u, (uint32_t)DERR_SELECT_OVERFLOW);
        desc[i] = (off << 8) | d;
      }
      __syncthreads();
      if (tid == 0) sm.run += total;
      // fill: warp per superblock of this chunk
      for (uint64_t j = warp; j < (uint64_t)BT && i0 + j < nsb; j += BNW) {
        const uint64_t si = i0 + j;
        const uint64_t dd = desc[si];
        const uint64_t poff = dd >> 8;
        const uint32_t wdt = (uint32_t)(dd & 127);
        if (poff + ((dd >> 7) & 1 ? 64ull * wdt : wdt) > pool_cap) continue;
        if (!((dd >> 7) & 1)) {
          const uint32_t start = t_b ? __ldcg(samples + 64 * si) : __ldcg(samples + samp_last - 64 * si);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t e = lane + 32 * h;
            const uint64_t k = 4096 * si + 64 * (uint64_t)e;
            uint64_t ent = 0;  // entries past the arg count stay zero; their samples do not exist
            if (k < m) {
              const uint32_t sp = t_b ? __ldcg(samples + 64 * si + e) : __ldcg(samples + samp_last - (64 * si + e));
              ent = (uint64_t)(uint32_t)(sp - start);
            }
            sm.ent[warp][e] = ent;
          }
          __syncwarp();
          if (lane < wdt) pool[poff + lane] = packed_word(lane, wdt, 64, [&](uint64_t e) { return sm.ent[warp][e]; });
          __syncwarp();
        } else {
          const uint64_t plo = __ldcg(st + si) >> 9;
          const uint64_t phi = ((si + 1 < nsb) ? __ldcg(en + si) : last - 1) >> 9;
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
    for (uint64_t q = tid; q < sb_nwords; q += BT)
      sbw[q] = packed_word(q, logn, nsb, [&](uint64_t i) { return __ldcg(st + i); });
    __syncthreads();
    if (tid == 0) {
      info[4 + (1 - t_b)] = sm.run;
      info[6 + (1 - t_b)] = sm.nlong;
    }
    __syncthreads();
  }
}

template <int IPT>
__global__ void __launch_bounds__(BT, 3) batch_build_kernel(BatchArgs a) {
  __shared__ BatchSmem sm;
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_fence_init();
    const uint32_t q = atomicAdd(a.queue, 1u);
    sm.item[1] = q < a.nitems ? a.items[q] : make_uint4(0, 0xFFFFFFFFu, 0, 0);
  }
  __syncthreads();
  uint32_t phases = 0;  // bit b: parity of staging buffer b's next completion
  for (;;) {
    const uint4 it = sm.item[1];
    __syncthreads();
    if (it.y == 0xFFFFFFFFu) break;
    if (threadIdx.x == 0) {  // take the next item while this one runs
      sm.item[0] = it;
      const uint32_t q = atomicAdd(a.queue, 1u);
      sm.item[1] = q < a.nitems ? a.items[q] : make_uint4(0, 0xFFFFFFFFu, 0, 0);
    }
    const uint32_t t = it.x, kind = it.y & 0xFF, level = it.y >> 8, tile = it.z;
    const uint64_t n = a.so[t + 1] - a.so[t];
    const uint32_t J = (uint32_t)(a.hb[t + 1] - a.hb[t]);
    if (kind == IT_H) {
      batch_h_item(a, t, tile, sm);
    } else if (kind == IT_W) {
      batch_wait(&a.done[4 * t + DN_HREADY], 1, a.err);
      switch (a.L) {
        case 1: batch_w_item<IPT, 1>(a, t, (int)level, tile, sm, phases); break;
        case 2: batch_w_item<IPT, 2>(a, t, (int)level, tile, sm, phases); break;
        case 3: batch_w_item<IPT, 3>(a, t, (int)level, tile, sm, phases); break;
        default: batch_w_item<IPT, 4>(a, t, (int)level, tile, sm, phases); break;
      }
    } else if (kind == IT_R) {
      batch_wait(&a.done[4 * t + DN_W], (uint32_t)a.L * J, a.err);
      batch_r_item(a, t, tile, sm);
    } else {
      batch_wait(&a.done[4 * t + DN_R], (uint32_t)(a.rb[t + 1] - a.rb[t]), a.err);
      batch_s_item(a, t, sm);
    }
    (void)n;
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host

struct BatchVariant {
  int ipt;       // symbols per thread per chunk (chunk = BT * ipt symbols)
  int cpt;       // chunks per H / W tile
  void (*kernel)(BatchArgs);
  uint64_t tile() const { return (uint64_t)BT * ipt * cpt; }
};

static const BatchVariant kBatchVariants[] = {
    {4, 4, batch_build_kernel<4>},   {4, 8, batch_build_kernel<4>},   {8, 2, batch_build_kernel<8>},
    {8, 4, batch_build_kernel<8>},   {8, 8, batch_build_kernel<8>},   {16, 2, batch_build_kernel<16>},
    {16, 4, batch_build_kernel<16>}, {16, 8, batch_build_kernel<16>},
};
constexpr int kNumBatchVariants = sizeof(kBatchVariants) / sizeof(kBatchVariants[0]);
constexpr uint64_t kMinTile = (uint64_t)BT * 4 * 4;  // the smallest tile of the variants

struct BatchImpl {
  uint64_t T = 0;
  int L = 0;
  uint32_t flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<uint64_t> n, so, bo, ro, sao, mo, deo, sbo, poo[2], rb;
  std::vector<uint32_t> order;  // texts by decreasing length
  uint64_t bits_words = 0, rank_words = 0, rtiles = 0;
  DevBuf in, d_so, d_bo, d_ro, d_sao, d_mo, d_deo, d_sbo, d_poo[2], d_rb, d_hb, d_items;
  DevBuf bits, rank, samples, marks, desc[2], sbw[2], pool[2], info, queue, err, thist, ttot, rstat, done;
  uint32_t nitems = 0;
  int items_variant = -1;  // the variant the uploaded items and H tiles follow
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

// The work list of one launch shape, in phase order (each phase's items by
// decreasing text length), and the texts' first H tiles.
static int batch_items(BatchImpl& b, int variant) {
  int rc;
  if (b.items_variant == variant) return WTG_OK;
  const uint64_t tile = kBatchVariants[variant].tile();
  const bool supports = (b.flags & (WTG_RANK | WTG_SELECT1 | WTG_SELECT0)) != 0;
  const bool sel = (b.flags & (WTG_SELECT1 | WTG_SELECT0)) != 0;
  std::vector<uint64_t> hb(b.T + 1, 0);
  for (uint64_t t = 0; t < b.T; ++t) hb[t + 1] = hb[t] + (b.n[t] + tile - 1) / tile;
  std::vector<uint4> items;
  items.reserve(hb[b.T] * (1 + b.L) + 2 * b.T + b.rtiles);
  for (uint32_t t : b.order)
    for (uint64_t j = 0; j < hb[t + 1] - hb[t]; ++j) items.push_back(make_uint4(t, IT_H, (uint32_t)j, 0));
  for (uint32_t t : b.order)
    for (int l = 0; l < b.L; ++l)
      for (uint64_t j = 0; j < hb[t + 1] - hb[t]; ++j)
        items.push_back(make_uint4(t, IT_W | ((uint32_t)l << 8), (uint32_t)j, 0));
  if (supports)
    for (uint32_t t : b.order)
      for (uint64_t r = 0; r < b.rb[t + 1] - b.rb[t]; ++r) items.push_back(make_uint4(t, IT_R, (uint32_t)r, 0));
  if (sel)
    for (uint32_t t : b.order) items.push_back(make_uint4(t, IT_S, 0, 0));
  if (items.size() >= 0xFFFFFFFFull) return fail(WTG_ERR_INVALID, "too many work items");
  cudaStream_t s = b.stream;
  if ((rc = b.d_items.ensure(std::max<size_t>(items.size(), 1) * sizeof(uint4), s))) return rc;
  if ((rc = b.d_hb.ensure((b.T + 1) * 8, s))) return rc;
  if (!items.empty())
    WTG_CK(cudaMemcpyAsync(b.d_items.p, items.data(), items.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(b.d_hb.p, hb.data(), (b.T + 1) * 8, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaStreamSynchronize(s));  // the host vectors must outlive the copies
  b.nitems = (uint32_t)items.size();
  b.items_variant = variant;
  return WTG_OK;
}

static BatchArgs batch_args(BatchImpl& b, int variant) {
  BatchArgs a;
  a.sym = b.in.as<uint8_t>();
  a.so = b.d_so.as<uint64_t>();
  a.T = b.T;
  a.L = b.L;
  a.flags = b.flags;
  a.tile = kBatchVariants[variant].tile();
  a.items = b.d_items.as<uint4>();
  a.nitems = b.nitems;
  a.hb = b.d_hb.as<uint64_t>();
  a.thist = b.thist.as<uint32_t>();
  a.ttot = b.ttot.as<uint32_t>();
  a.rb = b.d_rb.as<uint64_t>();
  a.rstat = b.rstat.as<uint64_t>();
  a.done = b.done.as<uint32_t>();
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

// every CTA of the persistent grid resident at once
static int batch_grid(const BatchVariant& v, uint32_t nitems) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.kernel, BT, 0);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t g = (uint64_t)std::max(1, per_sm) * (uint64_t)std::max(1, sms);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, std::max<uint32_t>(nitems, 1)));
}

// the whole build: clear the outputs, counters and the queue, run the
// persistent kernel (the item list of the variant is uploaded beforehand)
static int batch_enqueue(BatchImpl& b, int variant) {
  cudaStream_t s = b.stream;
  const BatchVariant& v = kBatchVariants[variant];
  WTG_CK(cudaMemsetAsync(b.bits.p, 0, b.bits_words * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(b.queue.p, 0, sizeof(uint32_t), s));
  WTG_CK(cudaMemsetAsync(b.done.p, 0, b.T * 4 * sizeof(uint32_t), s));
  WTG_CK(cudaMemsetAsync(b.rstat.p, 0, std::max<uint64_t>(b.rtiles, 1) * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(b.info.p, 0, b.T * 8 * sizeof(uint64_t), s));
  count_launch();
  v.kernel<<<batch_grid(v, b.nitems), BT, 0, s>>>(batch_args(b, variant));
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

BatchImpl* batch_new() { return new (std::nothrow) BatchImpl(); }

void batch_delete(BatchImpl* b) {
  if (!b) return;
  cudaStream_t s = b->stream;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  DevBuf* bufs[] = {&b->in,      &b->d_so,    &b->d_bo,    &b->d_ro,   &b->d_sao,  &b->d_mo,   &b->d_deo,
                    &b->d_sbo,   &b->d_poo[0], &b->d_poo[1], &b->d_rb,   &b->d_hb,   &b->d_items, &b->bits,
                    &b->rank,    &b->samples, &b->marks,   &b->desc[0], &b->desc[1], &b->sbw[0], &b->sbw[1],
                    &b->pool[0], &b->pool[1], &b->info,    &b->queue,  &b->err,    &b->thist,  &b->ttot,
                    &b->rstat,   &b->done};
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
  b.rb.assign(T + 1, 0);
  uint64_t max_htiles = 0;
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
    b.rb[t + 1] = b.rb[t] + ((W >> 3) + 1 + RT_SB - 1) / RT_SB;  // rank tiles of RT_SB superblocks
    max_htiles += (n + kMinTile - 1) / kMinTile;
  }
  b.bits_words = b.bo[T];
  b.rank_words = b.ro[T];
  b.rtiles = b.rb[T];
  b.order.resize(T);
  std::iota(b.order.begin(), b.order.end(), 0u);
  std::stable_sort(b.order.begin(), b.order.end(), [&](uint32_t x, uint32_t y) { return b.n[x] > b.n[y]; });
  b.items_variant = -1;

  auto up = [&](DevBuf& d, const void* h, size_t bytes) -> int {
    int r;
    if ((r = d.ensure(std::max<size_t>(bytes, 8), s))) return r;
    WTG_CK(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, s));
    return WTG_OK;
  };
  if ((rc = b.in.ensure(b.so[T] + 16, s))) return rc;
  if ((rc = up(b.d_so, b.so.data(), (T + 1) * 8))) return rc;
  if ((rc = up(b.d_rb, b.rb.data(), (T + 1) * 8))) return rc;
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
  if ((rc = b.thist.ensure(std::max<uint64_t>(max_htiles, 1) * BATCH_BINS * sizeof(uint32_t), s))) return rc;
  if ((rc = b.ttot.ensure(T * BATCH_BINS * sizeof(uint32_t), s))) return rc;
  if ((rc = b.rstat.ensure(std::max<uint64_t>(b.rtiles, 1) * sizeof(uint64_t), s))) return rc;
  if ((rc = b.done.ensure(T * 4 * sizeof(uint32_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(b.info.p, 0, T * 64, s));
  WTG_CK(cudaMemsetAsync(b.err.p, 0, 8, s));
  WTG_CK(cudaStreamSynchronize(s));  // the host vectors above must outlive the copies
  return WTG_OK;
}

// the build (clear, launch) captured once in a CUDA graph for replay
static int batch_capture(BatchImpl& b) {
  int rc;
  cudaStream_t s = b.stream;
  if ((rc = batch_items(b, b.variant))) return rc;
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
    if ((rc = batch_items(b, v))) break;
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

int batch_set_shape(BatchImpl& b, int tile, int ipt) {
  for (int v = 0; v < kNumBatchVariants; ++v) {
    if ((int)kBatchVariants[v].tile() == tile && kBatchVariants[v].ipt == ipt) {
      if (b.exec) cudaGraphExecDestroy(b.exec);
      if (b.graph) cudaGraphDestroy(b.graph);
      b.exec = nullptr;
      b.graph = nullptr;
      b.variant = v;
      return batch_capture(b);
    }
  }
  return fail(WTG_ERR_INVALID,
              "no such launch shape (symbols per tile / per thread: 4096/4, 8192/4, 4096/8, 8192/8, 16384/8, "
              "8192/16, 16384/16, 32768/16)");
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
  info[6] = b.variant >= 0 ? kBatchVariants[b.variant].tile() : 0;
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

int batch_tuning(const BatchImpl& b, int* tile, int* ipt, float* ms, int nms) {
  if (b.variant < 0) return fail(WTG_ERR_INVALID, "the batch has not run yet");
  *tile = (int)kBatchVariants[b.variant].tile();
  *ipt = kBatchVariants[b.variant].ipt;
  for (int v = 0; v < nms && v < kNumBatchVariants; ++v) ms[v] = b.tune_ms[v];
  return WTG_OK;
}

}  // namespace wtg
