// wtg_batch.cu -- batched builds: many independent texts, each with its own
// wavelet tree (level bitvector of L <= 4 levels), rank_support_v<1> and
// select_support_mcl<1>/<0>, all in one persistent launch.
//
// The reference builds one sequence per WT() call (levelWT/WT.C:43-227,
// driven by levelWT/WTTime.C:78-103); a batch there is a loop of calls.  Here
// one persistent kernel pulls work items from a device queue, made at plan
// time.  A text up to a size bound (at most its fair share of the batch: the
// total symbols over the resident CTAs) is one item:
//   X (text)              one CTA builds the whole text: every level's bits in
//                         one pass over the text (after a key histogram; for
//                         2 levels none: the level-1 key-1 run goes to a
//                         per-text stream and is moved into place once the
//                         key-0 count is known), the rank table and select
//                         marks a superblock per thread with the prefix
//                         carried over rounds, then select_support_mcl --
//                         no waits on other CTAs.
// A longer text is split over many CTAs, in phase order, each phase's items
// by decreasing text length:
//   H (text, tile)        the key histogram of one tile of the text;
//                         the text's last H item to finish turns the tiles'
//                         histograms into per-tile prefixes and totals
//   W (text, tile)        the tile's bits of every level
//   R (text, rank tile)   rank_support_v entries and select sample marks of
//                         256 superblocks, the ones before the tile from a
//                         decoupled look-back over the text's rank tiles
//                         (the reference layout and final-superblock rule)
//   S (text)              select_support_mcl, both polarities at once (a
//                         half block each): long/mini choice, widths, pool
//                         offsets (scan), mini blocks from the samples, long
//                         blocks by rank-table search, m_superblock packing.
// The split items come first, then the X items by decreasing length.  A
// split item first waits (bounded) until its text's previous phase is
// complete: per-text counters, bumped after each item's writes are fenced.
// Every item waits only on items taken from the queue before it, by CTAs
// that are running, so the launch always completes.  Data another CTA wrote
// is read through L2 (ld.cg, or bulk copies).
//
// Level bits.  Level l of a text is the text stably sorted by the top l bits
// of its symbols (levelWT/WT.C:118-190), so the symbols of (level l, key k)
// form one contiguous run starting at l*n + (symbols whose key is below k),
// and a range's piece of it starts after the earlier ranges' members.  A
// chunk of the text is staged in shared memory by cp.async.bulk; a lane
// takes one or two rows of 32 symbols.  For 1-2 levels the lane reads its
// own rows' bytes, forms each bit plane by a multiply-gather (level 0 is the
// top plane) and compresses the level-1 bits of each key by a nibble table;
// for 3-4 levels a warp takes 32 rows a lane per symbol: one ballot per bit
// plane and row, and for level l >= 1 each lane's place in the row stably
// sorted by key (lanes of smaller keys plus lanes before it with its key,
// from the planes by logic ops and popcounts), one OR-reduction of
// bit << place giving the row's sorted level word.  The lanes then count
// each key's members per row, scan them across the rows, and the CTA places
// the warps' pieces after one exchange per chunk.  A warp's piece of a key
// is assembled in shared memory from the rows' segments and stored: the
// words inside it plainly, its first and last word (shared with
// neighbouring pieces) with 32-bit atomic ORs on the zeroed bitvector.
// Every output has the layout of the single-sequence build.  The pool region
// of each text is sized by a bound that holds for any input (see plan), so
// the layout is fixed by the text lengths alone.  The first run times the
// candidate shapes (symbols per thread x split tile and whole-text bound)
// on the batch itself; the memsets plus the launch of the fastest are
// captured in a CUDA graph that later runs replay.

#include <algorithm>
#include <numeric>
#include <vector>

#include "wtg_internal.cuh"
#include "wtg_select.cuh"

namespace wtg {

WTG_WAIT_LIMIT_SETTER(batch)

constexpr int BATCH_LMAX = 4;
constexpr int BATCH_BINS = 1 << BATCH_LMAX;
constexpr int BATCH_NS = (1 << BATCH_LMAX) - 2;  // (level >= 1, key) slots: level l, key k is slot 2^l - 2 + k
constexpr int BATCH_NP = BATCH_NS / 2;           // slot pairs (two 16-bit counts in a word)
constexpr int BT = 256;                          // threads per CTA
constexpr int BNW = BT / 32;                     // warps per CTA
constexpr int ROWS = 32;                         // rows of 32 symbols per warp per chunk
constexpr int WSYM = ROWS * 32;                  // symbols per warp per chunk (one row per lane)
constexpr int CH = BNW * WSYM;                   // symbols per chunk (one row per lane)
constexpr int RPL_MAX = 2;                       // rows of 32 symbols per lane, at most
constexpr int CH_MAX = CH * RPL_MAX;
constexpr int RT_ITER = 8;                       // rows of BT words per rank tile
constexpr int RT_SB = RT_ITER * BT / 8;          // superblocks per rank tile

// work item: x = text, y = kind, z = tile
enum : uint32_t { IT_H = 0, IT_W = 1, IT_R = 2, IT_S = 3, IT_X = 4 };
// per-text completion counters of split texts: done[4 t + DN_*]
enum : uint32_t { DN_H = 0, DN_HREADY = 1, DN_W = 2, DN_R = 3 };

struct BatchArgs {
  const uint8_t* sym;     // concatenated texts
  const uint64_t* so;     // symbol offset of each text, T + 1
  uint64_t T;
  int L;
  uint32_t flags;
  uint64_t tile;          // symbols per H / W tile of a split text (a multiple of CH)
  const uint4* items;
  uint32_t nitems;
  const uint64_t* hb;     // first H tile of each text, T + 1 (split texts only have tiles)
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
  uint32_t* kstream;       // 2 levels: per text, the level-1 key-1 run of a whole text before it is moved
  const uint64_t* ko;      // its word offset per text
  uint32_t* queue;
  uint32_t* err;
};

struct BatchSmem {
  uint4 item[2];  // the item being processed and the next one (taken early)
  uint32_t hist[BATCH_BINS];
  uint32_t part[16][BATCH_BINS];
  uint64_t wbase[BATCH_NS];           // where the range's members of each slot start
  uint32_t wcnt[2][BNW][BATCH_NP];    // per chunk parity and warp: members per slot pair
  uint32_t scr[BNW][68];              // per warp: a piece being assembled (zero between uses)
  uint32_t flag;
  uint32_t sb[RT_SB];
  uint32_t lastw[2];  // rank tile: last word + 1 holding a one / a zero
  uint32_t wsum32[BNW];
  uint8_t lut[256 * 8];  // lut[byte * 8 + r] = position of the r-th set bit of byte
  uint16_t ctab[256];    // nibble compress table (compress32_tab)
  uint64_t prefix;
  uint64_t ent[BNW][64];
  uint64_t sdesc[BT];  // select pass: descriptors of the chunk's superblocks (a half block each)
  uint64_t hwsum[2][BNW / 2];  // select pass: per half, its warps' sums
  uint32_t wend[BATCH_NS];  // level pass: where each slot's run ended
  // two staging buffers for chunks of up to CH_MAX symbols (plus the text's
  // offset from a 16-byte boundary and the last lane's over-read), filled by
  // cp.async.bulk
  alignas(16) uint8_t stage[2][CH_MAX + 32];
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

// Adds the key histogram (bins 1 .. 2^L - 1) of cnt symbols at `in` to
// sm.hist (zeroed by the caller; a barrier before reading it).  The order of
// the symbols does not matter here, so each thread reads 16 at a time and
// counts the low-L-bit values of a 32-bit word bit-sliced (L <= 2) or
// bytewise (L = 3, 4); bin 0 is what remains.
__device__ void batch_count(const uint8_t* __restrict__ in, uint64_t cnt, int L, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t nbin = 1u << L, vmask = nbin - 1;
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
  for (; q + 3 * BT < nvec; q += 4 * BT) {  // four 16-byte loads in flight per thread
    uint4 u[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) u[h] = __ldg(vin + q + h * BT);
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      count_word(u[h].x); count_word(u[h].y); count_word(u[h].z); count_word(u[h].w);
    }
  }
  for (; q < nvec; q += BT) {
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

// level of slot s (slots of level l: 2^l - 2 .. 2^(l+1) - 3)
__host__ __device__ constexpr int slot_level(int s) { return s < 2 ? 1 : (s < 6 ? 2 : 3); }

// ---- H item: the key histogram of symbols [c0, c1) of a split text
__device__ void batch_h_item(const BatchArgs& a, uint32_t t, uint32_t j, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x;
  const int L = a.L;
  const uint32_t nbin = 1u << L;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint64_t c0 = (uint64_t)j * a.tile, c1 = min(n, c0 + a.tile), cnt = c1 - c0;
  if (tid < BATCH_BINS) sm.hist[tid] = 0;
  __syncthreads();
  batch_count(a.sym + a.so[t] + c0, cnt, L, sm);
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

// Bits of x at the set bits of m, packed to the low end in order
// ("compress"), by nibbles from a table: entry (m4 << 4) | x4 holds the kept
// bits of nibble x4 under mask nibble m4, and (bit 8 up) 2^(bits kept).
// Each nibble's bits land at the running product of those powers: one
// shared load and two multiply-adds per nibble, off the integer logic pipe
// (the logic-op form of Warren, Hacker's Delight, 2nd ed., section 7-4,
// takes five rounds of about 17 ops).
__device__ __forceinline__ uint32_t compress32_tab(uint32_t x, uint32_t m, const uint16_t* __restrict__ tab) {
  const uint32_t lo = (x & 0x0F0F0F0Fu) | ((m & 0x0F0F0F0Fu) << 4);
  const uint32_t hi = ((x >> 4) & 0x0F0F0F0Fu) | (m & 0xF0F0F0F0u);
  uint32_t res = 0, mult = 1;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t v = tab[(((i & 1) ? hi : lo) >> (8 * (i >> 1))) & 0xFFu];
    res += (v & 0xFFu) * mult;
    mult *= v >> 8;
  }
  return res;
}

// the compress table: thread i (< 256) fills entry i
__device__ __forceinline__ void compress_tab_init(uint16_t* tab) {
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
    const uint32_t m4 = i >> 4, x4 = i & 15u;
    uint32_t r = 0, k = 0;
    for (uint32_t b = 0; b < 4; ++b)
      if ((m4 >> b) & 1u) r |= ((x4 >> b) & 1u) << k++;
    tab[i] = (uint16_t)(r | ((1u << k) << 8));
  }
}

// Bit J of each of 32 bytes (w[k] holds bytes 4k .. 4k + 3) as one word.
// Per byte pair of words, a = the J-th bits of w[k] (at bits 0, 8, 16, 24)
// and b those of w[k + 1] moved up by 4: the product with 0x01020408 lifts
// a's four bits to bits 24..27 and b's to 28..31 (every other partial
// product lands once below bit 24, so no carry reaches them).
template <int J>
__device__ __forceinline__ uint32_t byte_plane(const uint32_t* w) {
  uint32_t p = 0;
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    const uint32_t a = (w[k] >> J) & 0x01010101u, b = (w[k + 1] >> J) & 0x01010101u;
    p |= (((a + (b << 4)) * 0x01020408u) >> 24) << (4 * k);
  }
  return p;
}

// Lane r's own rows (RPL rows of 32 symbols from symbol 32 RPL r of the
// warp's part of the chunk, staged at byte off + 32 RPL r of the warp's
// 16-byte aligned stage region st16) as 8 RPL words of four symbols: 2 RPL + 1
// aligned 16-byte loads, then a funnel shift by the offset.
template <int Q, int RPL>
__device__ __forceinline__ void batch_row_words(const uint8_t* __restrict__ st16, uint32_t lane, uint32_t sh,
                                                uint32_t (&w)[8 * RPL]) {
  const uint4* p = reinterpret_cast<const uint4*>(st16 + 32 * RPL * lane);
  uint32_t u[8 * RPL + 4];
#pragma unroll
  for (int v = 0; v < 2 * RPL + 1; ++v) {
    const uint4 q = p[v];
    u[4 * v] = q.x;
    u[4 * v + 1] = q.y;
    u[4 * v + 2] = q.z;
    u[4 * v + 3] = q.w;
  }
#pragma unroll
  for (int k = 0; k < 8 * RPL; ++k) w[k] = __funnelshift_r(u[k + Q], u[k + Q + 1], sh);
}

// Lane r's rows for 1 or 2 levels (rs = the first row's first symbol): per
// row its level-0 word w0 (the top plane, valid symbols only) and, for two
// levels, per key the members (cs) and level-1 bits (seg, compressed to the
// low end, the rows' bits one after another).
template <int LL, int RPL>
__device__ __forceinline__ void batch_row_swar(const uint8_t* __restrict__ st16, uint32_t off, uint64_t rs,
                                               uint64_t ce, uint32_t lane, const uint16_t* __restrict__ ctab,
                                               uint32_t (&w0)[RPL], uint32_t (&cs)[2], uint64_t (&seg)[2]) {
  uint32_t w[8 * RPL];
  const uint32_t sh = 8 * (off & 3);
  switch (off >> 2) {
    case 0: batch_row_words<0, RPL>(st16, lane, sh, w); break;
    case 1: batch_row_words<1, RPL>(st16, lane, sh, w); break;
    case 2: batch_row_words<2, RPL>(st16, lane, sh, w); break;
    default: batch_row_words<3, RPL>(st16, lane, sh, w); break;
  }
  cs[0] = cs[1] = 0;
  seg[0] = seg[1] = 0;
#pragma unroll
  for (int h = 0; h < RPL; ++h) {
    const uint64_t r = rs + 32 * h;
    const uint64_t left = r < ce ? ce - r : 0;
    const uint32_t V = left >= 32 ? 0xffffffffu : (1u << (uint32_t)left) - 1u;
    if constexpr (LL == 1) {
      w0[h] = byte_plane<0>(w + 8 * h) & V;
    } else {
      const uint32_t p1 = byte_plane<1>(w + 8 * h) & V, p0 = byte_plane<0>(w + 8 * h);
      w0[h] = p1;
      const uint32_t m0 = V & ~p1;
      seg[0] |= (uint64_t)compress32_tab(p0, m0, ctab) << cs[0];
      seg[1] |= (uint64_t)compress32_tab(p0, p1, ctab) << cs[1];
      cs[0] += __popc(m0);
      cs[1] += __popc(p1);
    }
  }
}

// One chunk's rows of a warp (lane = symbol, row r = symbols r0 + 32 r ..):
// lane r gets row r's bit planes kP, valid lanes kV, and level words kW
// (kW[0] = the top plane; kW[l] = the level-l bits of the row stably sorted
// by the l-bit key).
template <int LL, bool FULL>
__device__ __forceinline__ void batch_rows(const uint8_t* __restrict__ st, uint64_t r0, uint64_t ce, uint32_t lane,
                                           uint32_t (&kP)[LL], uint32_t& kV, uint32_t (&kW)[LL]) {
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const bool valid = FULL || r0 + 32 * r + lane < ce;
    const uint32_t x = valid ? (uint32_t)st[32 * r + lane] : 0u;
    uint32_t P[LL], W[LL];
#pragma unroll
    for (int j = 0; j < LL; ++j) P[j] = __ballot_sync(0xffffffffu, (x >> j) & 1u);
    const uint32_t V = FULL ? 0xffffffffu : __ballot_sync(0xffffffffu, valid);
    W[0] = P[LL - 1];
    // E: valid lanes whose key so far equals this lane's; less: valid lanes
    // whose key so far is smaller
    uint32_t E = V, less = 0;
#pragma unroll
    for (int l = 1; l < LL; ++l) {
      const int j = LL - l;  // the key bit level l adds
      const uint32_t m = 0u - ((x >> j) & 1u);
      less += __popc(E & ~P[j] & m);
      E &= ~(P[j] ^ m);
      const uint32_t place = less + __popc(E & lt);
      W[l] = __reduce_or_sync(0xffffffffu, ((x >> (LL - 1 - l)) & 1u) << place);
    }
    if (lane == (uint32_t)r) {
#pragma unroll
      for (int j = 0; j < LL; ++j) {
        kP[j] = P[j];
        kW[j] = W[j];
      }
      kV = V;
    }
  }
}

// Stages the chunk of text t at symbol c (up to ce) into staging buffer buf
// (thread 0): from the 16-byte boundary at or below the chunk -- the input has
// 16 bytes of padding after the last text, so the rounded-up tail stays inside
// it; chunk starts are multiples of 16 apart, so every chunk of a text has the
// same offset from its boundary.
__device__ __forceinline__ void batch_stage(BatchSmem& sm, const uint8_t* in, uint64_t c, uint64_t ce, int buf,
                                            uint32_t chunk) {
  const uint32_t off = (uint32_t)((uintptr_t)in & 15u);
  const uint64_t cnt = min((uint64_t)chunk, ce - c);
  const uint32_t bytes = (uint32_t)((off + cnt + 15) & ~15ull);
  fence_proxy_async_smem();
  mbar_expect_tx(&sm.bar[buf], bytes);
  bulk_g2s(sm.stage[buf], in + c - off, bytes, &sm.bar[buf]);
}

// The level bits of symbols [cb, ce) of text t (cb a multiple of the chunk,
// RPL rows of 32 symbols per lane: CH RPL symbols), every level in one pass; sm.wbase[s] (set before a barrier) is where the range's
// first member of slot s goes, and sm.wend[s] gets where its run ended.
// Chunks are staged two ahead; `staged`: the caller has already staged the
// first two.  slot1, if given, takes slot 1's run (positions from its own
// bit 0) in place of the text's bits.
template <int LL, int RPL>
__device__ void batch_w_range(const BatchArgs& a, uint32_t t, uint64_t cb, uint64_t ce, BatchSmem& sm,
                              uint32_t& phases, bool staged, uint32_t* __restrict__ slot1 = nullptr) {
  constexpr int NSL = (1 << LL) - 2;  // slots of levels >= 1
  constexpr int NP = (NSL + 1) / 2;   // their pairs
  constexpr int WS = WSYM * RPL;      // symbols per warp per chunk
  constexpr uint32_t CHR = CH * RPL;  // symbols per chunk
  static_assert(RPL == 1 || LL <= 2, "two rows per lane only for 1-2 levels");
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint8_t* __restrict__ in = a.sym + a.so[t];
  uint32_t* __restrict__ bits32 = reinterpret_cast<uint32_t*>(a.bits + a.bo[t]);
  uint32_t* __restrict__ scr = sm.scr[warp];
  // lane s < NSL: where the next chunk's members of slot s start (a text's
  // bits are below 2^31)
  uint32_t run = 0;
  if (NSL > 0 && lane < (uint32_t)NSL) run = (uint32_t)sm.wbase[lane];
  const uint32_t off = (uint32_t)((uintptr_t)in & 15u);
  if (tid == 0 && !staged) {
    if (cb < ce) batch_stage(sm, in, cb, ce, 0, CHR);
    if (cb + CHR < ce) batch_stage(sm, in, cb + CHR, ce, 1, CHR);
  }
  int cur = 0;
  for (uint64_t c0 = cb; c0 < ce; c0 += CHR, cur ^= 1) {
    mbar_wait(&sm.bar[cur], (phases >> cur) & 1u, a.err);
    phases ^= 1u << cur;
    const uint64_t r0 = c0 + (uint64_t)warp * WS;
    // lane r: its rows' level-0 words, and per slot their members (cs) and
    // level bits compressed to the low end (seg)
    uint32_t w0[RPL], cs[NSL > 0 ? NSL : 2];
    uint64_t seg[NSL > 0 ? NSL : 2];
    if constexpr (LL <= 2) {
      batch_row_swar<LL, RPL>(sm.stage[cur] + warp * WS, off, r0 + 32 * RPL * lane, ce, lane, sm.ctab, w0, cs, seg);
    } else {
      const uint8_t* const st = sm.stage[cur] + off + warp * WS;
      uint32_t kP[LL], kV = 0, kW[LL];
#pragma unroll
      for (int j = 0; j < LL; ++j) kP[j] = kW[j] = 0;
      if (c0 + CH <= ce) batch_rows<LL, true>(st, r0, ce, lane, kP, kV, kW);
      else batch_rows<LL, false>(st, r0, ce, lane, kP, kV, kW);
      w0[0] = kW[0];
      uint32_t M[NSL];
      M[0] = kV & ~kP[LL - 1];
      M[1] = kV & kP[LL - 1];
#pragma unroll
      for (int l = 2; l < LL; ++l)
#pragma unroll
        for (int k = 0; k < (1 << l); ++k)
          M[(1 << l) - 2 + k] = M[(1 << (l - 1)) - 2 + (k >> 1)] & ((k & 1) ? kP[LL - l] : ~kP[LL - l]);
#pragma unroll
      for (int l = 1; l < LL; ++l) {
        uint32_t acc = 0;  // where the key's segment starts in the row's sorted level word
#pragma unroll
        for (int k = 0; k < (1 << l); ++k) {
          const int q = (1 << l) - 2 + k;
          cs[q] = __popc(M[q]);
          seg[q] = cs[q] == 32 ? kW[l] : (kW[l] >> acc) & ((1u << cs[q]) - 1u);
          acc += cs[q];
        }
      }
    }
    // row prefixes (rp) and warp totals (tot) per slot, two 16-bit counts per scan
    uint32_t rp[NP > 0 ? NP : 1], tot[NP > 0 ? NP : 1];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const uint32_t v = cs[2 * p] | ((2 * p + 1 < NSL) ? (cs[2 * p + 1] << 16) : 0u);
      uint32_t inc = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t q = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += q;
      }
      rp[p] = inc - v;
      tot[p] = __shfl_sync(0xffffffffu, inc, 31);
      if (lane == 31) sm.wcnt[cur][warp][p] = inc;
    }
    // level 0: the rows' bits in order; a row reaching past the text's end
    // shares its word with level 1
#pragma unroll
    for (int h = 0; h < RPL; ++h) {
      const uint64_t rs = r0 + 32 * (RPL * lane + h);
      if (rs < ce) {
        if (rs + 32 <= n) bits32[rs >> 5] = w0[h];
        else if (w0[h]) atomicOr(bits32 + (rs >> 5), w0[h]);
      }
    }
    __syncthreads();  // the chunk's counts are in; every warp has read the staging buffer
    if (tid == 0 && c0 + 2 * CHR < ce) batch_stage(sm, in, c0 + 2 * CHR, ce, cur, CHR);
    if constexpr (NSL > 0) {
      uint32_t before[NP], all[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        uint32_t b = 0, s = 0;
#pragma unroll
        for (int w = 0; w < BNW; ++w) {
          const uint32_t x = sm.wcnt[cur][w][p];
          b += (w < (int)warp) ? x : 0u;
          s += x;
        }
        before[p] = b;
        all[p] = s;
      }
#pragma unroll
      for (int s = 0; s < NSL; ++s) {
        const uint32_t sh = (s & 1) ? 16 : 0;
        const uint32_t Ts = (tot[s >> 1] >> sh) & 0xFFFFu;
        if (Ts == 0) continue;
        const uint32_t d0 = __shfl_sync(0xffffffffu, run, s) + ((before[s >> 1] >> sh) & 0xFFFFu);
        const uint32_t c = cs[s];
        if (c) {
          const uint32_t d = d0 + ((rp[s >> 1] >> sh) & 0xFFFFu);
          const uint32_t q = (d >> 5) - (d0 >> 5), o = d & 31u;
          const uint64_t v = seg[s] << o;  // c <= 32 RPL bits from bit o: up to three words
          atomicOr(scr + q, (uint32_t)v);
          if (o + c > 32) atomicOr(scr + q + 1, (uint32_t)(v >> 32));
          if (RPL > 1 && o + c > 64) atomicOr(scr + q + 2, (uint32_t)(seg[s] >> (64 - o)));
        }
        __syncwarp();
        const uint32_t nw = ((d0 + Ts + 31) >> 5) - (d0 >> 5);
        for (uint32_t q = lane; q < nw; q += 32) {
          const uint32_t v = scr[q];
          scr[q] = 0;
          uint32_t* g = ((s == 1 && slot1) ? slot1 : bits32) + (d0 >> 5) + q;
          if (q == 0 || q + 1 == nw) {
            if (v) atomicOr(g, v);
          } else {
            *g = v;
          }
        }
        __syncwarp();
      }
      uint32_t mine = 0;
#pragma unroll
      for (int p = 0; p < NP; ++p)
        if ((lane >> 1) == (uint32_t)p) mine = ((lane & 1) ? (all[p] >> 16) : all[p]) & 0xFFFFu;
      run += mine;
    }
  }
  if (NSL > 0 && warp == 0 && lane < (uint32_t)NSL) sm.wend[lane] = run;
}

// ---- W item: every level's bits of tile j of a split text
template <int LL, int RPL>
__device__ void batch_w_item(const BatchArgs& a, uint32_t t, uint32_t j, BatchSmem& sm, uint32_t& phases) {
  constexpr int NSL = (1 << LL) - 2;
  const uint32_t tid = threadIdx.x;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint64_t cb = (uint64_t)j * a.tile, ce = min(n, cb + a.tile);
  // slot (l, k): l * n + symbols of keys below k + the earlier tiles' members of key k
  if (NSL > 0 && (int)tid < NSL) {
    const int l = slot_level((int)tid);
    const uint32_t k = tid - ((1u << l) - 2);
    const uint32_t* tot = a.ttot + (uint64_t)t * BATCH_BINS;
    const uint32_t* pre = a.thist + (a.hb[t] + j) * BATCH_BINS;
    uint64_t below = 0, mine = 0;
    for (uint32_t b = 0; b < (1u << LL); ++b) {
      const uint32_t key = b >> (LL - l);
      if (key < k) below += __ldcg(tot + b);
      if (key == k) mine += __ldcg(pre + b);
    }
    sm.wbase[tid] = (uint64_t)l * n + below + mine;
  }
  __syncthreads();
  batch_w_range<LL, RPL>(a, t, cb, ce, sm, phases, false);
  batch_signal(&a.done[4 * t + DN_W]);
}

// Select marks of word wi of a batch text (its bits are below 2^31, so
// every position and count fits 32 bits): the same marks as word_marks() in
// wtg_select.cuh -- for select1 (x) and select0 (~x) every 64th arg, every
// superblock start (arg 4096q) and end (arg 4096q + 4095).  K1 = ones before
// the word; the next multiple of 64 is d1 = (-K1) & 63 ones into it and
// d0 = K1 & 63 zeros into it, so one select serves both polarities.
__device__ __forceinline__ void batch_word_marks(uint64_t x, uint32_t c, uint32_t K1, uint32_t wi, uint64_t zmask,
                                                 bool sel1, bool sel0, uint32_t* __restrict__ samples,
                                                 uint32_t samp_last, uint64_t* __restrict__ starts1,
                                                 uint64_t* __restrict__ starts0, uint64_t* __restrict__ ends1,
                                                 uint64_t* __restrict__ ends0, uint32_t& lastw1, uint32_t& lastw0) {
  const uint64_t z = ~x & zmask;
  const uint32_t cz = __popcll(z);
  const uint32_t base = wi << 6;
  const uint32_t K0 = base - K1;
  const uint32_t d1 = (0u - K1) & 63u, d0 = K1 & 63u;
  const bool s1 = sel1 && d1 < c, s0 = sel0 && d0 < cz;
  if (s1 || s0) {
    const uint32_t pos = base + sel64_0(s1 ? x : z, s1 ? d1 : d0);
    if (s1) {
      const uint32_t k = K1 + d1;
      samples[k >> 6] = pos;
      if ((k & 4095) == 0) starts1[k >> 12] = pos;
    }
    if (s0) {
      const uint32_t pos0 = s1 ? base + (uint32_t)(__ffsll((long long)z) - 1) : pos;
      const uint32_t k = K0 + d0;
      samples[samp_last - (k >> 6)] = pos0;
      if ((k & 4095) == 0) starts0[k >> 12] = pos0;
    }
  }
  if (sel1) {
    const uint32_t e = 4095u - (K1 & 4095u);
    if (e < c) ends1[(K1 + e) >> 12] = base + sel64_0(x, e);
    lastw1 = c ? wi + 1 : lastw1;
  }
  if (sel0) {
    const uint32_t e = 4095u - (K0 & 4095u);
    if (e < cz) ends0[(K0 + e) >> 12] = base + sel64_0(z, e);
    lastw0 = cz ? wi + 1 : lastw0;
  }
}

// ---- R item: rank tile r (RT_SB superblocks) of a split text's bitvector:
// rank_support_v entries and select marks.  The ones before the tile come
// from a decoupled look-back over the text's rank tiles (the R items are
// taken from the queue in order, so every predecessor has started).  The
// tile holding the final superblock writes the arg counts; last args go to
// the text's info.
__device__ void batch_r_tile(const BatchArgs& a, uint32_t t, uint32_t r, BatchSmem& sm) {
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
  // rows of BT words the tile needs: through the word of the final
  // superblock's entry (word 8 NB, past the data when W is a multiple of 8)
  const uint64_t wend = max(W, 8 * NB + 1);
  const int nrows = (int)min((uint64_t)RT_ITER, (wend - wbase + BT - 1) / BT);
  if (tid < 2) sm.lastw[tid] = 0;
  uint64_t w[RT_ITER];
  uint32_t c[RT_ITER], inc[RT_ITER];
#pragma unroll
  for (int i = 0; i < RT_ITER; ++i) {
    if (i >= nrows) {
      w[i] = 0;
      c[i] = inc[i] = 0;
      if (g8 == 7) sm.sb[i * (BT / 8) + warp * 4 + (lane >> 3)] = 0;
      continue;
    }
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
  const uint32_t tprefix = (uint32_t)sm.prefix;  // a text's bits are below 2^31
  const uint32_t r_last = (uint32_t)(W - 8 * NB);  // words of the final superblock
  const uint32_t W32 = (uint32_t)W, NB32 = (uint32_t)NB, slast = (uint32_t)samp_last;
  uint32_t last1 = 0, last0 = 0;
#pragma unroll
  for (int i = 0; i < RT_ITER; ++i) {
    if (i >= nrows) break;
    const uint32_t sbl = i * (BT / 8) + warp * 4 + (lane >> 3);
    const uint32_t b = r * RT_SB + sbl;  // superblock
    const uint32_t wi = (uint32_t)wbase + i * BT + tid;
    const uint32_t sb_before = tprefix + sm.sb[sbl];
    const uint32_t excl = inc[i] - c[i];
    const uint32_t sbt = __shfl_sync(0xffffffffu, inc[i], (lane & ~7u) + 7);
    if (flags & WTG_RANK) {
      // field k (1..7) = count before block k; the final superblock writes
      // only fields 1..max(r,1), r = its words (rank_support_v_par.hpp:99-108)
      const uint32_t kmax = (b < NB32) ? 7u : (r_last > 1 ? r_last : 1u);
      uint64_t part = (g8 >= 1 && g8 <= kmax) ? ((uint64_t)excl << (63 - 9 * g8)) : 0ull;
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) part |= __shfl_xor_sync(0xffffffffu, part, o);
      if (g8 == 0 && b <= NB32) {
        rank[2 * (uint64_t)b] = sb_before;
        rank[2 * (uint64_t)b + 1] = part;
      }
    }
    if (b == NB32 && g8 == 0) {
      info[0] = sb_before + sbt;
      info[1] = size - (sb_before + sbt);
    }
    if (wi < W32)
      batch_word_marks(w[i], c[i], sb_before + excl, wi, wi == W32 - 1 ? tailmask : ~0ull, sel1, sel0, samples,
                       slast, starts1, starts0, ends1, ends0, last1, last0);
  }
  // the tile's last word holding a one / a zero (word indices < 2^26), then
  // the position after its last one / zero, once per tile
  const uint32_t l1 = __reduce_max_sync(0xffffffffu, last1);
  const uint32_t l0 = __reduce_max_sync(0xffffffffu, last0);
  if (lane == 0) {
    if (l1) atomicMax(&sm.lastw[0], l1);
    if (l0) atomicMax(&sm.lastw[1], l0);
  }
  __syncthreads();
  if (tid < 2 && sm.lastw[tid]) {
    const uint64_t e = last_arg_end(words, sm.lastw[tid], W, tailmask, 1 - (int)tid);
    atomicMax((unsigned long long*)&info[2 + tid], (unsigned long long)e);
  }
  batch_signal(&a.done[4 * t + DN_R]);
}

// ---- S item: select_support_mcl of both polarities of one text, at once:
// warps 0-3 build select1, warps 4-7 select0, each half with its own named
// barrier and scan, so that a text pays the phase's latency chain once
__device__ __forceinline__ void batch_half_sync(uint32_t half) {
  static_assert(BT == 256, "named barriers of 128 threads");
  if (half) asm volatile("bar.sync 2, 128;" ::: "memory");  // constant ids: ptxas reserves barriers 0-2 only
  else asm volatile("bar.sync 1, 128;" ::: "memory");
}

// exclusive scan of one u64 per thread over a half block; the half's total
// through *total
__device__ __forceinline__ uint64_t half_excl_scan(uint64_t v, uint32_t half, BatchSmem& sm, uint64_t* total) {
  const uint32_t lane = threadIdx.x & 31, hwarp = (threadIdx.x >> 5) & 3;
  uint64_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  if (lane == 31) sm.hwsum[half][hwarp] = inc;
  batch_half_sync(half);
  uint64_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    const uint64_t x = sm.hwsum[half][w];
    before += (w < (int)hwarp) ? x : 0;
    all += x;
  }
  batch_half_sync(half);
  *total = all;
  return before + inc - v;
}

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
  constexpr uint32_t HT = BT / 2, HNW = BNW / 2;  // threads and warps per half
  const uint32_t half = warp >> 2, htid = tid & (HT - 1), hwarp = warp & (HNW - 1);
  const int t_b = half ? 0 : 1;
  if (t_b ? sel1 : sel0) {
    const uint64_t m = t_b ? m1 : m0;
    const uint64_t nsb = (m + 4095) >> 12;
    const uint64_t last = t_b ? last1 : last0;
    const uint64_t* __restrict__ st = t_b ? starts1 : starts0;
    const uint64_t* __restrict__ en = t_b ? ends1 : ends0;
    uint64_t* __restrict__ desc = a.desc[t_b] + a.deo[t];
    uint64_t* __restrict__ pool = a.pool[t_b] + a.poo[t_b][t];
    const uint64_t pool_cap = a.poo[t_b][t + 1] - a.poo[t_b][t];
    uint64_t* __restrict__ sdesc = sm.sdesc + half * HT;
    uint64_t run = 0;  // pool words of the chunks before (the same in every thread of the half)
    uint32_t nlong = 0;
    for (uint64_t i0 = 0; i0 < nsb; i0 += HT) {
      const uint64_t i = i0 + htid;
      uint64_t sz = 0, d = 0;
      if (i < nsb) {
        const uint64_t start = __ldcg(st + i);
        const uint64_t end = (i + 1 < nsb) ? __ldcg(en + i) : last - 1;
        const uint64_t span = end - start;
        const uint64_t lng = span > logn4;
        const uint64_t wdt = lng ? hi64(end) + 1 : hi64(span) + 1;
        d = (lng << 7) | wdt;
        sz = lng ? 64 * wdt : wdt;
      }
      nlong += __popc(__ballot_sync(0xffffffffu, (d >> 7) & 1));  // per warp; summed below
      uint64_t total;
      const uint64_t off = run + half_excl_scan(sz, half, sm, &total);
      if (i < nsb) {
        if (off + sz > pool_cap) atomicCAS(a.err, 0u, (uint32_t)DERR_SELECT_OVERFLOW);
        desc[i] = (off << 8) | d;
        sdesc[htid] = (off << 8) | d;
      }
      batch_half_sync(half);
      run += total;
      // fill: warp per superblock of this chunk
      for (uint64_t j = hwarp; j < (uint64_t)HT && i0 + j < nsb; j += HNW) {
        const uint64_t si = i0 + j;
        const uint64_t dd = sdesc[j];
        const uint64_t poff = dd >> 8;
        const uint32_t wdt = (uint32_t)(dd & 127);
        if (poff + ((dd >> 7) & 1 ? 64ull * wdt : wdt) > pool_cap) continue;
        if (!((dd >> 7) & 1)) {
          // the superblock's samples (every 64th arg), relative to its first
          // (entry 0, arg 4096 si < m): one round of loads
          uint32_t sp[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t e = lane + 32 * h;
            const uint64_t k = 4096 * si + 64 * (uint64_t)e;
            sp[h] = k < m ? (t_b ? __ldcg(samples + 64 * si + e) : __ldcg(samples + samp_last - (64 * si + e))) : 0u;
          }
          const uint32_t start = __shfl_sync(0xffffffffu, sp[0], 0);
          // the block is exactly wdt words (64 entries of wdt bits, wdt <= 32
          // for a mini block): zero them, OR each entry in at bit e * wdt as
          // 32-bit halves (a half and perhaps the next), then store
          uint32_t* blk = reinterpret_cast<uint32_t*>(sm.ent[warp]);
          if (lane < wdt) blk[2 * lane] = blk[2 * lane + 1] = 0;
          __syncwarp();
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t e = lane + 32 * h;
            const uint64_t k = 4096 * si + 64 * (uint64_t)e;
            // entries past the arg count stay zero; their samples do not exist
            const uint64_t val = k < m ? (uint64_t)(uint32_t)(sp[h] - start) : 0ull;
            const uint32_t bit = e * wdt, wq = bit >> 5, sh = bit & 31u;
            if (val) {
              atomicOr(blk + wq, (uint32_t)(val << sh));
              if (sh + wdt > 32) atomicOr(blk + wq + 1, (uint32_t)(val >> (32 - sh)));
            }
          }
          __syncwarp();
          if (lane < wdt) pool[poff + lane] = (uint64_t)blk[2 * lane] | ((uint64_t)blk[2 * lane + 1] << 32);
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
      batch_half_sync(half);  // sdesc is the next chunk's
    }
    // m_superblock
    uint64_t* __restrict__ sbw = a.sbw[t_b] + a.sbo[t];
    const uint64_t sb_nwords = (nsb * logn + 63) / 64;
    for (uint64_t q = htid; q < sb_nwords; q += HT)
      sbw[q] = packed_word(q, logn, nsb, [&](uint64_t i) { return __ldcg(st + i); });
    // long superblocks: every warp of the half counted its lanes' chunks
    if (lane == 0) sm.hwsum[half][hwarp] = nlong;
    batch_half_sync(half);
    if (htid == 0) {
      uint64_t nl = 0;
      for (int w = 0; w < (int)HNW; ++w) nl += sm.hwsum[half][w];
      info[4 + (1 - t_b)] = run;
      info[6 + (1 - t_b)] = nl;
    }
  }
  __syncthreads();
}

// ---- the rank table and select marks of a whole text in this CTA (its bits
// were written by this CTA): a thread per 512-bit superblock, BT
// superblocks per round; the ones before a superblock from a block scan of
// the round's superblock counts plus the rounds before.  Per word at most
// one in-word select (the next 64th one or zero: the select1 samples of a
// superblock are consecutive from index ceil(ones before / 64), the select0
// samples descend from the back from ceil(zeros before / 64)); superblock
// ends (at most one per polarity in 512 bits) and the last args once per
// superblock.  A text's bits are below 2^31: 32-bit positions and counts.
__device__ void batch_r_whole(const BatchArgs& a, uint32_t t, BatchSmem& sm) {
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint32_t size = (uint32_t)((uint64_t)a.L * n);
  const uint32_t W = (size + 63) / 64, NB = W >> 3;
  const uint32_t r_last = W - 8 * NB;  // words of the final superblock
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  const uint32_t flags = a.flags;
  const bool sel1 = flags & WTG_SELECT1, sel0 = flags & WTG_SELECT0, sel = sel1 || sel0;
  const uint64_t* __restrict__ words = a.bits + a.bo[t];
  uint64_t* __restrict__ rank = a.rank + a.ro[t];
  uint32_t* __restrict__ samples = a.samples + a.sao[t];
  const uint32_t samp_last = W + 1;
  const uint64_t nsbc = size / 4096 + 2;
  uint64_t* __restrict__ starts1 = a.marks + a.mo[t];
  uint64_t* __restrict__ starts0 = starts1 + nsbc;
  uint64_t* __restrict__ ends1 = starts0 + nsbc;
  uint64_t* __restrict__ ends0 = ends1 + nsbc;
  uint64_t* __restrict__ info = a.info + 8 * (uint64_t)t;
  const uint8_t* __restrict__ lut = sm.lut;
  if (tid < 2) sm.lastw[tid] = 0;
  uint32_t carry = 0;                       // ones before the round
  uint32_t last_sb1 = ~0u, last_sb0 = ~0u;  // last superblocks holding a one / a zero
  for (uint32_t b0 = 0; b0 <= NB; b0 += BT) {
    const uint32_t b = b0 + tid;  // this thread's superblock
    const bool live = b <= NB;
    const bool tail = 8 * b + 8 >= W;  // holds the last data word, or lies past it
    uint64_t w[8];
    if (!tail) {
      const ulonglong2* p = reinterpret_cast<const ulonglong2*>(words + 8 * (uint64_t)b);
      const ulonglong2 q0 = __ldcg(p), q1 = __ldcg(p + 1), q2 = __ldcg(p + 2), q3 = __ldcg(p + 3);
      w[0] = q0.x; w[1] = q0.y; w[2] = q1.x; w[3] = q1.y; w[4] = q2.x; w[5] = q2.y; w[6] = q3.x; w[7] = q3.y;
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t wi = 8 * b + j;
        w[j] = (live && wi < W) ? (__ldcg(words + wi) & (wi == W - 1 ? tailmask : ~0ull)) : 0ull;
      }
    }
    uint32_t cnt[8], tot = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      cnt[j] = __popcll(w[j]);
      tot += cnt[j];
    }
    // block exclusive scan of the superblock counts
    uint32_t inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t q = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (uint32_t)o) inc += q;
    }
    if (lane == 31) sm.wsum32[warp] = inc;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int v = 0; v < BNW; ++v) {
      const uint32_t x = sm.wsum32[v];
      before += v < (int)warp ? x : 0u;
      all += x;
    }
    __syncthreads();
    const uint32_t sb_before = carry + before + inc - tot;  // ones before the superblock
    carry += all;
    if (!live) continue;
    const uint32_t bits_in = tail ? (size > 512 * b ? min(512u, size - 512 * b) : 0u) : 512u;  // its data bits
    const uint32_t zb = 512 * b - sb_before;                 // zeros before it
    uint32_t* __restrict__ p1 = samples + ((sb_before + 63) >> 6);
    uint32_t* __restrict__ p0 = samples + (samp_last - ((zb + 63) >> 6));
    uint32_t excl = 0, n1 = 0, n0 = 0;
    uint64_t part = 0;
    const uint32_t kmax = b < NB ? 7u : (r_last > 1 ? r_last : 1u);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t x = w[j];
      const uint32_t cj = cnt[j];
      if (j && (uint32_t)j <= kmax) part |= (uint64_t)excl << (63 - 9 * j);
      if (sel) {
        const uint32_t vb = tail ? min(64u, (uint32_t)max(0, (int)(size - 512 * b - 64 * j))) : 64u;
        const uint32_t czj = vb - cj;  // zeros of the word's data bits
        const uint32_t cl = __popc((uint32_t)x);
        const uint32_t K1 = sb_before + excl, K0 = zb + 64u * j - excl;
        const uint32_t d1 = (0u - K1) & 63u, d0 = K1 & 63u;
        const bool s1 = sel1 && d1 < cj, s0 = sel0 && d0 < czj;
        const uint32_t off = sel64_lut(s1 ? x : ~x, s1 ? d1 : d0, s1 ? cl : 32u - cl, lut);
        // both polarities only when K1 % 64 == 0: the word's first one and first zero
        const uint32_t off0 = s1 ? (uint32_t)(__ffsll((long long)~x) - 1) : off;
        const uint32_t pos = 512 * b + 64u * j;
        if (s1) p1[n1] = pos + off;
        if (s0) *(p0 - n0) = pos + off0;
        if (s1 && ((K1 + d1) & 4095u) == 0) starts1[(K1 + d1) >> 12] = pos + off;
        if (s0 && ((K0 + d0) & 4095u) == 0) starts0[(K0 + d0) >> 12] = pos + off0;
        n1 += s1;
        n0 += s0;
      }
      excl += cj;
    }
    if (flags & WTG_RANK) reinterpret_cast<ulonglong2*>(rank)[b] = make_ulonglong2(sb_before, part);
    if (b == NB) {
      info[0] = sb_before + excl;
      info[1] = size - (sb_before + excl);
    }
    if (sel) {
      // superblock ends: arg 4095 of a 4096-arg superblock, at most one per
      // polarity in 512 bits; the rare superblock that ends one of each takes
      // a second round
      const uint32_t cz = bits_in - excl;
      const uint32_t e1 = 4095u - (sb_before & 4095u), e0 = 4095u - (zb & 4095u);
      bool h1 = sel1 && e1 < excl, h0 = sel0 && e0 < cz;
      const uint32_t act = __activemask();
      while (__any_sync(act, h1 || h0)) {
        const bool t1 = h1;
        const uint32_t e = t1 ? e1 : e0;
        uint32_t bef = 0, r = 0, jj = 0;
        uint64_t xx = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const uint32_t vb = tail ? min(64u, (uint32_t)max(0, (int)(size - 512 * b - 64 * j))) : 64u;
          const uint32_t cj = t1 ? cnt[j] : vb - cnt[j];
          const bool here = bef <= e && e < bef + cj;
          xx = here ? w[j] : xx;
          r = here ? e - bef : r;
          jj = here ? (uint32_t)j : jj;
          bef += cj;
        }
        xx = t1 ? xx : ~xx;
        const uint32_t pos = 512 * b + 64 * jj + sel64_lut(xx, r, __popc((uint32_t)xx), lut);
        if (h1) ends1[(sb_before + e1) >> 12] = pos;
        else if (h0) ends0[(zb + e0) >> 12] = pos;
        if (h1) h1 = false;
        else h0 = false;
      }
      last_sb1 = excl ? b : last_sb1;
      last_sb0 = cz ? b : last_sb0;
    }
  }
  if (sel) {
    // position after the last one / zero: the last word holding one in the
    // last superblock holding one
    uint32_t e[2] = {0, 0};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint32_t sb = q == 0 ? last_sb1 : last_sb0;
      if (sb == ~0u) continue;
      for (int j = 7; j >= 0; --j) {
        const uint32_t wi = 8 * sb + j;
        if (wi >= W) continue;
        uint64_t x = __ldcg(words + wi);
        if (q) x = ~x & (wi == W - 1 ? tailmask : ~0ull);
        if (x) {
          e[q] = (wi << 6) + hi64(x) + 1;
          break;
        }
      }
    }
    const uint32_t m1 = __reduce_max_sync(0xffffffffu, e[0]), m0 = __reduce_max_sync(0xffffffffu, e[1]);
    if (lane == 0) {
      if (m1) atomicMax(&sm.lastw[0], m1);
      if (m0) atomicMax(&sm.lastw[1], m0);
    }
  }
  __syncthreads();
  if (tid < 2 && sel) info[2 + tid] = sm.lastw[tid];
  __syncthreads();  // the select pass reads the arg counts and last args next
}

// ---- X item: the whole text t in this CTA
template <int L, int RPL>
__device__ void batch_x_item(const BatchArgs& a, uint32_t t, BatchSmem& sm, uint32_t& phases) {
  const uint32_t tid = threadIdx.x;
  const uint64_t n = a.so[t + 1] - a.so[t];
  const uint8_t* in = a.sym + a.so[t];
  if (tid == 0) {  // the level pass's first chunks load while the histogram runs
    if (n > 0) batch_stage(sm, in, 0, n, 0, CH * RPL);
    if (n > CH * RPL) batch_stage(sm, in, CH * RPL, n, 1, CH * RPL);
  }
  if constexpr (L == 2) {
    // no histogram: level 1's key-0 run starts at n; the key-1 run (at n + the
    // key-0 members, unknown until the pass ends) goes to the text's stream
    // from its bit 0 and is moved into place after the pass
    uint32_t* __restrict__ ks = a.kstream + a.ko[t];
    const uint64_t kw = (n + 31) / 32 + 1;
    for (uint64_t i = tid; i < kw; i += BT) ks[i] = 0;
    if (tid == 0) {
      sm.wbase[0] = n;
      sm.wbase[1] = 0;
    }
    __syncthreads();
    batch_w_range<2, RPL>(a, t, 0, n, sm, phases, true, ks);
    __syncthreads();
    // move the key-1 run (m bits) to bit p = n + (key-0 members) of the text:
    // word j of the bits takes the stream's bits from 32 j - p on
    const uint32_t p = sm.wend[0], m = (uint32_t)(2 * n) - p;
    uint32_t* __restrict__ bits32 = reinterpret_cast<uint32_t*>(a.bits + a.bo[t]);
    if (m > 0) {
      const uint32_t j0 = p >> 5, j1 = (p + m - 1) >> 5, o = p & 31u;
      for (uint32_t j = j0 + tid; j <= j1; j += BT) {
        const uint32_t q = j - j0;
        const uint32_t hi = __ldcg(ks + q), lo = q ? __ldcg(ks + q - 1) : 0u;
        const uint32_t v = o ? ((hi << o) | (lo >> (32 - o))) : hi;
        if (j == j0) bits32[j] |= v;  // its low bits are key 0's (or level 0's)
        else bits32[j] = v;
      }
    }
  } else {
    if (tid < BATCH_BINS) sm.hist[tid] = 0;
    __syncthreads();
    batch_count(in, n, L, sm);
    __syncthreads();
    // slot (l, k): level l starts at l * n, key k after the symbols of smaller keys
    constexpr int NSL = (1 << L) - 2;
    if (NSL > 0 && (int)tid < NSL) {
      const int l = slot_level((int)tid);
      const uint32_t k = tid - ((1u << l) - 2);
      uint64_t below = 0, others = 0;
      for (uint32_t b = 1; b < (1u << L); ++b) {
        others += sm.hist[b];
        if ((b >> (L - l)) < k) below += sm.hist[b];
      }
      if (k > 0) below += n - others;  // bin 0 has key 0
      sm.wbase[tid] = (uint64_t)l * n + below;
    }
    __syncthreads();
    batch_w_range<L, RPL>(a, t, 0, n, sm, phases, true);
  }
  __syncthreads();  // the bits are written (read back through L2 below)
  if (a.flags & WTG_RANK) batch_r_whole(a, t, sm);
  if (a.flags & (WTG_SELECT1 | WTG_SELECT0)) batch_s_item(a, t, sm);
}

// one instantiation per level count (the level pass keeps per-slot state in
// registers) and rows per lane
template <int LL, int RPL>
__global__ void __launch_bounds__(BT, LL == 4 ? 2 : 3) batch_build_kernel(BatchArgs a) {
  __shared__ BatchSmem sm;
  for (uint32_t i = threadIdx.x; i < BNW * 68; i += BT) (&sm.scr[0][0])[i] = 0;
  sel_lut_init(sm.lut);
  compress_tab_init(sm.ctab);
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
    const uint32_t t = it.x, kind = it.y, tile = it.z;
    const uint32_t J = (uint32_t)(a.hb[t + 1] - a.hb[t]);
    if (kind == IT_X) {
      batch_x_item<LL, RPL>(a, t, sm, phases);
    } else if (kind == IT_H) {
      batch_h_item(a, t, tile, sm);
    } else if (kind == IT_W) {
      batch_wait(&a.done[4 * t + DN_HREADY], 1, a.err);
      batch_w_item<LL, RPL>(a, t, tile, sm, phases);
    } else if (kind == IT_R) {
      batch_wait(&a.done[4 * t + DN_W], J, a.err);
      batch_r_tile(a, t, tile, sm);
    } else {
      batch_wait(&a.done[4 * t + DN_R], (uint32_t)(a.rb[t + 1] - a.rb[t]), a.err);
      batch_s_item(a, t, sm);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host

struct BatchImpl {
  uint64_t T = 0;
  int L = 0;
  uint32_t flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<uint64_t> n, so, bo, ro, sao, mo, deo, sbo, poo[2], rb, ko;
  std::vector<uint32_t> order;  // texts by decreasing length
  uint64_t bits_words = 0, rank_words = 0, rtiles = 0;
  DevBuf in, d_so, d_bo, d_ro, d_sao, d_mo, d_deo, d_sbo, d_poo[2], d_rb, d_hb, d_items;
  DevBuf bits, rank, samples, marks, desc[2], sbw[2], pool[2], info, queue, err, thist, ttot, rstat, done;
  DevBuf kstream, d_ko;
  uint32_t nitems = 0;
  bool items_valid = false;
  uint64_t tile = 65536;      // symbols per H / W tile of a split text
  int64_t whole_req = -1;     // texts up to this many symbols are X items (-1: automatic)
  int rpl = 1;                // rows of 32 symbols per lane in the level pass
  bool shape_fixed = false;   // set_shape was called: no tuning
  uint64_t whole_max = 0;     // the bound in use
  uint64_t nwhole = 0;        // texts built whole
  uint64_t items_tile = 0;    // the shape the uploaded items follow
  int64_t items_whole = -2;
  float tune_ms[8] = {0};
  std::vector<uint64_t> h_info;
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

static void (*batch_kernel(int L, int rpl))(BatchArgs) {
  switch (L) {
    case 1: return rpl == 2 ? batch_build_kernel<1, 2> : batch_build_kernel<1, 1>;
    case 2: return rpl == 2 ? batch_build_kernel<2, 2> : batch_build_kernel<2, 1>;
    case 3: return batch_build_kernel<3, 1>;
    default: return batch_build_kernel<4, 1>;
  }
}

// CTAs of the persistent grid: every one resident at once
static int batch_grid_size(int L, int rpl) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel(L, rpl), BT, 0);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, per_sm) * std::max(1, sms);
}

// The work list: split texts' items in phase order (each phase by decreasing
// text length), then one X item per other text by decreasing length; and the
// split texts' first H tiles.  A text is built whole when it holds at most
// the bound: by default its fair share of the batch (the total over the
// resident CTAs), at least 65536 symbols.
static int batch_items(BatchImpl& b) {
  int rc;
  if (b.items_valid && b.items_tile == b.tile && b.items_whole == b.whole_req) return WTG_OK;
  const uint64_t total = b.so[b.T];
  b.whole_max = b.whole_req >= 0 ? (uint64_t)b.whole_req
                                 : std::max<uint64_t>(65536, total / (uint64_t)batch_grid_size(b.L, 1));
  const uint64_t tile = b.tile;
  const bool supports = (b.flags & (WTG_RANK | WTG_SELECT1 | WTG_SELECT0)) != 0;
  const bool sel = (b.flags & (WTG_SELECT1 | WTG_SELECT0)) != 0;
  std::vector<uint64_t> hb(b.T + 1, 0);
  std::vector<uint32_t> split, whole;
  for (uint32_t t : b.order) (b.n[t] > b.whole_max ? split : whole).push_back(t);
  for (uint64_t t = 0; t < b.T; ++t) hb[t + 1] = hb[t] + (b.n[t] > b.whole_max ? (b.n[t] + tile - 1) / tile : 0);
  std::vector<uint4> items;
  items.reserve(hb[b.T] * 2 + 2 * b.T + b.rtiles);
  for (uint32_t t : split)
    for (uint64_t j = 0; j < hb[t + 1] - hb[t]; ++j) items.push_back(make_uint4(t, IT_H, (uint32_t)j, 0));
  for (uint32_t t : split)
    for (uint64_t j = 0; j < hb[t + 1] - hb[t]; ++j) items.push_back(make_uint4(t, IT_W, (uint32_t)j, 0));
  if (supports)
    for (uint32_t t : split)
      for (uint64_t r = 0; r < b.rb[t + 1] - b.rb[t]; ++r) items.push_back(make_uint4(t, IT_R, (uint32_t)r, 0));
  if (sel)
    for (uint32_t t : split) items.push_back(make_uint4(t, IT_S, 0, 0));
  for (uint32_t t : whole) items.push_back(make_uint4(t, IT_X, 0, 0));
  if (items.size() >= 0xFFFFFFFFull) return fail(WTG_ERR_INVALID, "too many work items");
  cudaStream_t s = b.stream;
  if ((rc = b.d_items.ensure(std::max<size_t>(items.size(), 1) * sizeof(uint4), s))) return rc;
  if ((rc = b.d_hb.ensure((b.T + 1) * 8, s))) return rc;
  if ((rc = b.thist.ensure(std::max<uint64_t>(hb[b.T], 1) * BATCH_BINS * sizeof(uint32_t), s))) return rc;
  if (!items.empty())
    WTG_CK(cudaMemcpyAsync(b.d_items.p, items.data(), items.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(b.d_hb.p, hb.data(), (b.T + 1) * 8, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaStreamSynchronize(s));  // the host vectors must outlive the copies
  b.nitems = (uint32_t)items.size();
  b.nwhole = whole.size();
  b.items_valid = true;
  b.items_tile = b.tile;
  b.items_whole = b.whole_req;
  return WTG_OK;
}

static BatchArgs batch_args(BatchImpl& b) {
  BatchArgs a;
  a.sym = b.in.as<uint8_t>();
  a.so = b.d_so.as<uint64_t>();
  a.T = b.T;
  a.L = b.L;
  a.flags = b.flags;
  a.tile = b.tile;
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
  a.kstream = b.kstream.as<uint32_t>();
  a.ko = b.d_ko.as<uint64_t>();
  a.queue = b.queue.as<uint32_t>();
  a.err = b.err.as<uint32_t>();
  return a;
}

// the whole build: clear the outputs, counters and the queue, run the
// persistent kernel (the item list is uploaded beforehand)
static int batch_enqueue(BatchImpl& b) {
  cudaStream_t s = b.stream;
  WTG_CK(cudaMemsetAsync(b.bits.p, 0, b.bits_words * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(b.queue.p, 0, sizeof(uint32_t), s));
  WTG_CK(cudaMemsetAsync(b.done.p, 0, b.T * 4 * sizeof(uint32_t), s));
  WTG_CK(cudaMemsetAsync(b.rstat.p, 0, std::max<uint64_t>(b.rtiles, 1) * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(b.info.p, 0, b.T * 8 * sizeof(uint64_t), s));
  count_launch();
  const int grid = (int)std::min<uint64_t>((uint64_t)batch_grid_size(b.L, b.rpl), std::max<uint32_t>(b.nitems, 1));
  batch_kernel(b.L, b.rpl)<<<grid, BT, 0, s>>>(batch_args(b));
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
                    &b->rstat,   &b->done,    &b->kstream, &b->d_ko};
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
  b.ko.assign(T + 1, 0);
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
    // 2 levels: the whole-text pass's key-1 stream, n bits and a zero word (in 32-bit words)
    b.ko[t + 1] = b.ko[t] + (L == 2 ? (n + 31) / 32 + 1 : 0);
    b.rb[t + 1] = b.rb[t] + ((W >> 3) + 1 + RT_SB - 1) / RT_SB;  // rank tiles of RT_SB superblocks
  }
  b.bits_words = b.bo[T];
  b.rank_words = b.ro[T];
  b.rtiles = b.rb[T];
  b.order.resize(T);
  std::iota(b.order.begin(), b.order.end(), 0u);
  std::stable_sort(b.order.begin(), b.order.end(), [&](uint32_t x, uint32_t y) { return b.n[x] > b.n[y]; });
  b.items_valid = false;

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
  if ((rc = up(b.d_ko, b.ko.data(), (T + 1) * 8))) return rc;
  if ((rc = b.kstream.ensure(std::max<uint64_t>(b.ko[T], 2) * 4, s))) return rc;
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
  if ((rc = batch_items(b))) return rc;
  WTG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  rc = batch_enqueue(b);
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

// The autotuner's candidates: symbols per thread of the level pass (one or
// two 32-symbol rows per lane; two only for 1-2 levels) x (split tile,
// whole-text bound): the automatic bound, and every text split into tiles
// of 32768 or 131072 symbols.
struct BatchShape {
  int rpl;
  uint64_t tile;
  int64_t whole;
};
static const BatchShape kBatchShapes[] = {
    {1, 65536, -1}, {2, 65536, -1}, {1, 32768, 0}, {2, 32768, 0}, {1, 131072, 0}, {2, 131072, 0},
};
constexpr int kNumBatchShapes = sizeof(kBatchShapes) / sizeof(kBatchShapes[0]);

static void batch_drop_graph(BatchImpl& b) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.exec = nullptr;
  b.graph = nullptr;
}

// Times every candidate shape once (after one warm-up run) on the batch's
// own input and keeps the fastest.
static int batch_tune(BatchImpl& b) {
  int rc = WTG_OK;
  cudaStream_t s = b.stream;
  cudaEvent_t e0, e1;
  WTG_CK(cudaEventCreate(&e0));
  WTG_CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_v = 0;
  for (int v = 0; v < kNumBatchShapes; ++v) {
    b.tune_ms[v] = 0;
    if (kBatchShapes[v].rpl > 1 && b.L > 2) continue;
    b.rpl = kBatchShapes[v].rpl;
    b.tile = kBatchShapes[v].tile;
    b.whole_req = kBatchShapes[v].whole;
    if ((rc = batch_items(b))) break;
    if ((rc = batch_enqueue(b))) break;
    WTG_CK(cudaEventRecord(e0, s));
    if ((rc = batch_enqueue(b))) break;
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
  b.rpl = kBatchShapes[best_v].rpl;
  b.tile = kBatchShapes[best_v].tile;
  b.whole_req = kBatchShapes[best_v].whole;
  return WTG_OK;
}

int batch_set_shape(BatchImpl& b, int tile, int64_t whole_max, int symbols_per_thread) {
  if (symbols_per_thread != 32 && symbols_per_thread != 64)
    return fail(WTG_ERR_INVALID, "symbols_per_thread must be 32 or 64");
  if (symbols_per_thread == 64 && b.L > 2) return fail(WTG_ERR_INVALID, "64 symbols per thread need 1-2 levels");
  const int chunk = CH * (symbols_per_thread / 32);
  if (tile < chunk || tile > (1 << 24) || tile % chunk)
    return fail(WTG_ERR_INVALID, "tile must be a multiple of 256 x symbols_per_thread in that .. 2^24");
  if (whole_max < -1) return fail(WTG_ERR_INVALID, "whole_max must be -1 (automatic) or >= 0");
  batch_drop_graph(b);
  b.tile = (uint64_t)tile;
  b.whole_req = whole_max;
  b.rpl = symbols_per_thread / 32;
  b.shape_fixed = true;
  for (float& m : b.tune_ms) m = 0;
  return WTG_OK;
}

int batch_run(BatchImpl& b) {
  int rc;
  b.info_valid = false;
  if (!b.exec) {
    if (!b.shape_fixed && (rc = batch_tune(b))) return rc;
    if ((rc = batch_capture(b))) return rc;
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
  info[6] = b.tile;
  info[7] = b.n[t] <= b.whole_max ? 1 : 0;
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

int batch_shape(const BatchImpl& b, int* tile, int64_t* whole_max, int* symbols_per_thread, uint64_t* whole_texts,
                float* ms, int nms) {
  if (!b.items_valid) return fail(WTG_ERR_INVALID, "the batch has not run yet");
  *tile = (int)b.tile;
  *whole_max = (int64_t)b.whole_max;
  *symbols_per_thread = 32 * b.rpl;
  *whole_texts = b.nwhole;
  for (int v = 0; v < nms; ++v) ms[v] = v < kNumBatchShapes ? b.tune_ms[v] : 0.f;
  return WTG_OK;
}

}  // namespace wtg
