// wtg_lsel.cu -- select inside one level of a tree's bitvector: the plain
// select_support_mcl route and a learned index beside it.
//
// Plain: select_support_mcl<t_b> on the concatenated bitvector, offset by the
// args before the level (wt_int's per-level select step,
// wt_int/wt_int_par.hpp:651-656, with the whole level as the node).
//
// Learned (no counterpart in the reference).  For level l and polarity t_b
// let m be the level's args (ones for t_b = 1, zeros for t_b = 0).  Args
// 1..m are cut into segments of G = 2^g args, g the smallest with at most
// `segments` segments.  Segment j carries a line
//     pred(k) = base_j + floor(slope_j * x / 2^16),  x = k - 1 - j*G,
// fitted by least squares on (k, select(k)) pairs computed by the plain
// select (lsel_fit_kernel), and signed bounds dlo_j <= select(k) - pred(k)
// <= dhi_j that hold for EVERY k of the segment: lsel_bound_kernel derives
// them from each word's first and last arg and the rank table, so no pair is
// left unchecked.
//
// The window is searched through a rank directory small enough to stay in
// L2 (lsel_dir_kernel, from the rank_support_v table): per 8192-bit block of
// the concatenated bitvector the exact ones before it (u64), and per 512-bit
// superblock an int8 residual against the line between its block's two
// counts -- 24 bytes per 8192 bits.  A query reads its segment record, the
// block counts inside [pred + dlo, pred + dhi] (L2), its block's sixteen
// residuals (L2), which give the superblock exactly, and then the
// superblock's eight words: one 64-byte line from DRAM, where plain select
// reads a mini-block entry and then the data.  Segments whose window
// exceeds max_window, blocks whose residuals do not fit int8, and any search
// that does not close are answered by the plain select, so every answer is
// the plain select's answer.
#include <algorithm>
#include <vector>

#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {

struct LselLevel {
  uint64_t A;        // args of this polarity before the level start (global count)
  uint64_t m;        // args inside the level
  uint32_t g;        // log2 of args per segment
  uint32_t nseg;     // segments of this level
  uint64_t rec_off;  // index of the level's first segment record
  uint64_t off;      // the level's first bit in the concatenated bitvector
  uint64_t pad;
};

// segment record (uint4): x = base (level position), y = slope (16.16 fixed,
// positions per arg), z = dlo, w = dhi (int32)
struct LselImpl {
  TreeImpl* tree = nullptr;
  uint64_t tree_gen = 0;
  uint32_t segments = 0, samples = 0, max_window = 0;
  int L = 0;
  uint64_t n = 0;
  uint64_t nseg[2] = {0, 0};
  std::vector<LselLevel> lv_host[2];
  SelView plain_host[2];
  DevBuf lv[2], rec[2], plain[2], stats;  // plain: the SelView of the fallback
  DevBuf dbase, dres;                     // rank directory: block counts, superblock residuals
  uint64_t dblocks = 0;
};

namespace {

constexpr int LSEL_FRAC = 16;
constexpr int LSEL_MAX_PROBES = 40;
constexpr long long LSEL_SAT = 1ll << 30;
// stats words per polarity: fallback segments, max window, window sum, misses
constexpr int LSEL_ST = 4;
constexpr int LSEL_DIR_SB = 16;          // superblocks per directory block (8192 bits)
constexpr int8_t LSEL_DIR_OVER = -128;   // residual 0 of a block whose residuals do not fit int8

// L2 cache policies for the query's loads (per load, no device state): the
// index (segment records, directory) evict-last, the data lines evict-first
__device__ __forceinline__ uint64_t l2_policy_last() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t ld_u64_pol(const uint64_t* a, uint64_t pol) {
  uint64_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ uint4 ld_v4_pol(const void* a, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(a), "l"(pol));
  return v;
}
// one 32-byte sector (32-byte aligned) in a single load
__device__ __forceinline__ void ld_v4u64_pol(const void* a, uint64_t pol, uint64_t& x, uint64_t& y, uint64_t& z,
                                             uint64_t& w) {
  asm volatile("ld.global.nc.L2::cache_hint.v4.u64 {%0, %1, %2, %3}, [%4], %5;"
               : "=l"(x), "=l"(y), "=l"(z), "=l"(w)
               : "l"(a), "l"(pol));
}

__device__ __forceinline__ uint64_t lsel_pred(uint32_t base, uint32_t slope, uint64_t x) {
  return (uint64_t)base + (((uint64_t)slope * x) >> LSEL_FRAC);
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__device__ __forceinline__ int sat32(long long v) {
  return (int)(v < -LSEL_SAT ? -LSEL_SAT : (v > LSEL_SAT ? LSEL_SAT : v));
}

// ones before each level start: out[l] = rank1(l * n), l = 0..L
__global__ void level_args_kernel(const uint64_t* __restrict__ tbl, const uint64_t* __restrict__ words, uint64_t n,
                                  int L, uint64_t* __restrict__ out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l <= L) out[l] = rank1_dev(tbl, words, (uint64_t)l * n);
}

template <int T_B>
__global__ void level_select_kernel(SelView v, const uint64_t* __restrict__ la, uint64_t n, int L,
                                    const uint64_t* __restrict__ lev, const uint64_t* __restrict__ kq, uint64_t nq,
                                    uint64_t* __restrict__ out) {
  const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t l = lev[q], k = kq[q];
  uint64_t res = NONE64;
  if (l < (uint64_t)L) {
    const uint64_t off = l * n;
    const uint64_t o0 = __ldg(la + l), o1 = __ldg(la + l + 1);
    const uint64_t A = T_B ? o0 : off - o0;
    const uint64_t m = T_B ? o1 - o0 : n - (o1 - o0);
    if (k >= 1 && k <= m) {
      const uint64_t p = select_dev(v, A + k);
      res = p == NONE64 ? NONE64 : p - off;
    }
  }
  out[q] = res;
}

__device__ __forceinline__ int lsel_find_level(const LselLevel* __restrict__ lv, int L, uint64_t gs) {
  for (int l = 0; l < L; ++l)
    if (gs >= lv[l].rec_off && gs < lv[l].rec_off + lv[l].nseg) return l;
  return -1;
}

// Training: one warp per segment fits the line by least squares on `samples`
// evenly spaced (k, select(k)) pairs of the segment (all of them when the
// segment is shorter), computed with the plain select.
__global__ void lsel_fit_kernel(SelView v, const LselLevel* __restrict__ lv, int L, uint64_t n, uint32_t samples,
                                uint64_t nseg_total, uint4* __restrict__ rec) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t gs = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; gs < nseg_total; gs += warps) {
    const int l = lsel_find_level(lv, L, gs);
    if (l < 0) continue;  // warp-uniform
    const LselLevel d = lv[l];
    const uint64_t j = gs - d.rec_off;
    const uint64_t kS = 1 + (j << d.g);
    const uint64_t len = umin64((uint64_t)1 << d.g, d.m - (j << d.g));
    const uint64_t P = min((uint64_t)samples, len);
    const uint64_t off = (uint64_t)l * n;
    const uint64_t y0 = select_dev(v, d.A + kS) - off;
    double sx = 0, sy = 0, sxx = 0, sxy = 0;
    for (uint64_t i = lane; i < P; i += 32) {
      const uint64_t x = len > P ? (i * len) / P : i;
      const double y = (double)(select_dev(v, d.A + kS + x) - off - y0);
      const double xd = (double)x;
      sx += xd;
      sy += y;
      sxx += xd * xd;
      sxy += xd * y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xFFFFFFFFu, sx, o);
      sy += __shfl_xor_sync(0xFFFFFFFFu, sy, o);
      sxx += __shfl_xor_sync(0xFFFFFFFFu, sxx, o);
      sxy += __shfl_xor_sync(0xFFFFFFFFu, sxy, o);
    }
    if (lane == 0) {
      const double N = (double)P;
      const double mx = sx / N, my = sy / N;
      const double vx = sxx / N - mx * mx, cxy = sxy / N - mx * my;
      double slope = (P > 1 && vx > 0) ? cxy / vx : 0.0;
      if (!(slope > 0)) slope = 0;
      long long base = (long long)y0 + llrint(my - slope * mx);
      base = base < 0 ? 0 : (base > (long long)(n - 1) ? (long long)(n - 1) : base);
      const double sf = slope * (double)(1 << LSEL_FRAC);
      const uint32_t slope_fx = sf >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)llrint(sf);
      rec[gs] = make_uint4((uint32_t)base, slope_fx, 0x7FFFFFFFu, 0x80000000u);
    }
  }
}

// Exact error bounds.  For the args k in [kA, kB] of one word piece (the part
// of a word inside one level), positions rise strictly from the first arg qA
// to the last qB, so  qA + (k - kA) <= select(k) <= qB - (kB - k).  With
// pred(k) = base + floor(s x) and s x linear in k, the extremes of
// select(k) - pred(k) over a segment's sub-range lie at its two ends up to
// the floor's one unit:  dhi >= max(U(k1), U(k2)) + 1 and
// dlo <= min(D(k1), D(k2)) - 1, U and D the upper and lower position bounds
// minus pred.  Updates are combined per warp (lanes of a warp usually share a
// segment) before the atomics.
__global__ void lsel_bound_kernel(const uint64_t* __restrict__ words, const uint64_t* __restrict__ tbl, uint64_t n,
                                  int L, uint64_t total, double inv_n, const LselLevel* __restrict__ lv0,
                                  const LselLevel* __restrict__ lv1, uint4* __restrict__ rec0,
                                  uint4* __restrict__ rec1) {
  constexpr int SLOTS = 4;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwords = (total + 63) >> 6;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t wbase = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wbase < nwords;
       wbase += stride) {
    const uint64_t w = wbase + lane;
    uint64_t key[SLOTS];
    int slo[SLOTS], shi[SLOTS];
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
      key[t] = ~0ull;
      slo[t] = 0;
      shi[t] = 0;
    }
    int ns = 0;
    if (w < nwords) {
      const uint64_t word = words[w];
      const uint64_t p0 = w << 6, p1 = min(p0 + 64, total);
      const uint64_t r1w = rank1_dev(tbl, words, p0);
      uint64_t l = (uint64_t)((double)p0 * inv_n);
      while (l > 0 && l * n > p0) --l;
      while ((l + 1) * n <= p0) ++l;
      for (; l < (uint64_t)L; ++l) {
        const uint64_t ls = l * n;
        if (ls >= p1) break;
        const uint64_t a = max(p0, ls), b = min(p1, ls + n);
        const uint32_t sa = (uint32_t)(a - p0), sb = (uint32_t)(b - p0);
        const uint64_t mask = (sb >= 64 ? ~0ull : ((1ull << sb) - 1)) & (~0ull << sa);
        const uint64_t r1a = r1w + (sa ? __popcll(word & ((1ull << sa) - 1)) : 0);
        for (int t_b = 0; t_b < 2; ++t_b) {
          const LselLevel d = (t_b ? lv1 : lv0)[l];
          if (d.nseg == 0) continue;
          const uint64_t bits = (t_b ? word : ~word) & mask;
          const uint32_t c = __popcll(bits);
          if (!c) continue;
          const uint64_t Ra = t_b ? r1a : a - r1a;
          const uint64_t kA = Ra - d.A + 1, kB = kA + c - 1;
          const long long qA = (long long)(p0 + (uint64_t)(__ffsll((long long)bits) - 1) - ls);
          const long long qB = (long long)(p0 + (uint64_t)(63 - __clzll((long long)bits)) - ls);
          uint4* rec = t_b ? rec1 : rec0;
          for (uint64_t j = (kA - 1) >> d.g; j <= (kB - 1) >> d.g; ++j) {
            const uint64_t k1 = max(kA, 1 + (j << d.g)), k2 = min(kB, (j + 1) << d.g);
            const uint4 r = rec[d.rec_off + j];
            const long long e1 = (long long)lsel_pred(r.x, r.y, k1 - 1 - (j << d.g));
            const long long e2 = (long long)lsel_pred(r.x, r.y, k2 - 1 - (j << d.g));
            const long long U1 = qB - (long long)(kB - k1) - e1, U2 = qB - (long long)(kB - k2) - e2;
            const long long D1 = qA + (long long)(k1 - kA) - e1, D2 = qA + (long long)(k2 - kA) - e2;
            const int hi = sat32(max(U1, U2) + 1), lo = sat32(min(D1, D2) - 1);
            const uint64_t kk = ((uint64_t)t_b << 63) | (d.rec_off + j);
            bool placed = false;
#pragma unroll
            for (int t = 0; t < SLOTS; ++t)
              if (!placed && t == ns) {
                key[t] = kk;
                slo[t] = lo;
                shi[t] = hi;
                placed = true;
              }
            if (placed) {
              ++ns;
            } else {
              atomicMin((int*)&rec[d.rec_off + j].z, lo);
              atomicMax((int*)&rec[d.rec_off + j].w, hi);
            }
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < SLOTS; ++t) {
      const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key[t]);
      const int vlo = __reduce_min_sync(grp, slo[t]);
      const int vhi = __reduce_max_sync(grp, shi[t]);
      if (key[t] != ~0ull && lane == (uint32_t)(__ffs(grp) - 1)) {
        uint4* rec = (key[t] >> 63) ? rec1 : rec0;
        const uint64_t idx = key[t] & ~(1ull << 63);
        atomicMin((int*)&rec[idx].z, vlo);
        atomicMax((int*)&rec[idx].w, vhi);
      }
    }
  }
}

__global__ void lsel_stats_kernel(const uint4* __restrict__ rec, uint64_t nseg, uint32_t max_window,
                                  unsigned long long* __restrict__ st) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nseg) return;
  const uint4 r = rec[i];
  const long long win = (long long)(int)r.w - (long long)(int)r.z;
  if (win < 0 || win > (long long)max_window) {
    atomicAdd(st + 0, 1ull);
  } else {
    atomicMax(st + 1, (unsigned long long)win);
    atomicAdd(st + 2, (unsigned long long)win);
  }
}

// Rank directory: thread per block j of LSEL_DIR_SB superblocks: base[j] =
// ones before superblock 16 j, base[nblocks] = all ones (the rank table's
// last entry NB counts the ones before superblock NB, which still holds data
// when the words are not a multiple of 8: its words are added), res[j][i] =
// ones before superblock 16 j + i minus base[j] + floor((base[j + 1] -
// base[j]) i / 16).  Residual 0 is always 0; a block with a residual outside
// int8 stores LSEL_DIR_OVER there instead.
__global__ void lsel_dir_kernel(const uint64_t* __restrict__ tbl, const uint64_t* __restrict__ words, uint64_t W,
                                uint64_t nblocks, uint64_t* __restrict__ base, int8_t* __restrict__ res,
                                unsigned long long* __restrict__ over) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j > nblocks) return;
  const uint64_t NB = W >> 3;
  auto ones_before = [&](uint64_t sb) -> uint64_t {  // superblock sb <= NB, or all ones past it
    if (sb <= NB) return __ldg(tbl + 2 * sb);
    uint64_t c = __ldg(tbl + 2 * NB);
    for (uint64_t w = 8 * NB; w < W; ++w) c += __popcll(__ldg(words + w));
    return c;
  };
  const uint64_t b0 = ones_before(LSEL_DIR_SB * j);
  base[j] = b0;
  if (j == nblocks) return;
  const uint64_t b1 = ones_before(LSEL_DIR_SB * (j + 1));
  int8_t r[LSEL_DIR_SB];
  bool bad = false;
#pragma unroll
  for (int i = 0; i < LSEL_DIR_SB; ++i) {
    const uint64_t sb = LSEL_DIR_SB * j + i;
    long long d = 0;
    if (sb <= NB) d = (long long)__ldg(tbl + 2 * sb) - (long long)(b0 + (((b1 - b0) * (uint64_t)i) >> 4));
    bad = bad || d < -127 || d > 127;
    r[i] = (int8_t)d;
  }
  if (bad) {
    r[0] = LSEL_DIR_OVER;
    atomicAdd(over, 1ull);
  }
  int4* dst = reinterpret_cast<int4*>(res + LSEL_DIR_SB * j);
  *dst = *reinterpret_cast<const int4*>(r);
}

struct LselView {
  const uint64_t* words;
  const uint64_t* tbl;
  uint64_t nwords;  // data words of the concatenated bitvector
  uint64_t total;   // its bits
  const uint64_t* dbase;
  const int8_t* dres;
  uint64_t dblocks;
  uint64_t n;
  int L;
  uint32_t max_window;
  const LselLevel* lv;
  const uint4* rec;
  const SelView* plain;  // device copy
  unsigned long long* misses;
};

// the plain select_support_mcl answer; kept out of line so that its
// registers do not count against the learned search's occupancy
__device__ __noinline__ uint64_t lsel_plain(const SelView* v, uint64_t K, uint64_t off) {
  const uint64_t p = select_dev(*v, K);
  return p == NONE64 ? NONE64 : p - off;
}

// The learned search, NQ queries per thread taken stage by stage so that
// each stage's loads for all of them are in flight together: inputs; level
// and segment records; the window's directory block (counts and residuals);
// the superblock (branch-free binary search over the residuals) and its one
// 64-byte line; the word and the in-word select.  A query whose window
// exceeds max_window, whose block's residuals overflow, or whose search does
// not close is answered by the plain select, so every answer is the plain
// select's answer.
template <int T_B, int NQ>
__global__ void __launch_bounds__(256) lsel_query_kernel_nq(LselView v, const uint64_t* __restrict__ lev,
                                                            const uint64_t* __restrict__ kq, uint64_t nq,
                                                            uint64_t* __restrict__ out) {
  const uint64_t keep = l2_policy_last(), stream = l2_policy_first();
  const uint64_t q0 = (uint64_t)blockIdx.x * blockDim.x * NQ + threadIdx.x;
  uint64_t l[NQ], k[NQ], res[NQ];
  int st[NQ];  // 0 searching, 1 done, 2 fallback
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    const uint64_t q = q0 + (uint64_t)i * blockDim.x;
    st[i] = q < nq ? 0 : 1;
    l[i] = q < nq ? lev[q] : 0;
    k[i] = q < nq ? kq[q] : 0;
    res[i] = NONE64;
  }
  LselLevel d[NQ];
  uint4 r[NQ];
  uint64_t K[NQ];
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (st[i] == 0 && (l[i] >= (uint64_t)v.L)) st[i] = 1;
    if (st[i] == 0) {
      d[i] = v.lv[l[i]];
      if (k[i] == 0 || k[i] > d[i].m) st[i] = 1;
    }
    if (st[i] == 0) {
      K[i] = d[i].A + k[i];
      const uint64_t j = (k[i] - 1) >> d[i].g;
      r[i] = ld_v4_pol(v.rec + d[i].rec_off + j, keep);
    }
  }
  uint64_t b_lo[NQ], b_hi[NQ], c_lo[NQ], c_hi[NQ];
  uint4 rv[NQ];
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (st[i] != 0) continue;
    const int dlo = (int)r[i].z, dhi = (int)r[i].w;
    if (dhi < dlo || (uint32_t)(dhi - dlo) > v.max_window) {
      st[i] = 2;
      continue;
    }
    const uint64_t km = k[i] - 1, j = km >> d[i].g;
    const long long pred = (long long)r[i].x + (long long)(((uint64_t)r[i].y * (km - (j << d[i].g))) >> LSEL_FRAC);
    const long long lo = max(pred + dlo, 0ll), hi = min(pred + dhi, (long long)v.n - 1);
    b_lo[i] = (d[i].off + (uint64_t)lo) >> 13;
    b_hi[i] = (d[i].off + (uint64_t)hi) >> 13;
    if (b_hi[i] >= v.dblocks) b_hi[i] = v.dblocks - 1;
    if (b_lo[i] > b_hi[i]) b_lo[i] = b_hi[i];
    c_lo[i] = ld_u64_pol(v.dbase + b_lo[i], keep);
    c_hi[i] = ld_u64_pol(v.dbase + b_lo[i] + 1, keep);
    rv[i] = ld_v4_pol(reinterpret_cast<const uint4*>(v.dres) + b_lo[i], keep);
  }
  auto before = [&](uint64_t b, uint64_t ones) -> uint64_t {
    return T_B ? ones : umin64(b << 13, v.total) - ones;
  };
  uint64_t w0[NQ];
  uint32_t need[NQ];
  uint64_t wv[NQ][8];
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (st[i] != 0) continue;
    if (before(b_lo[i], c_lo[i]) >= K[i]) {
      atomicAdd(v.misses, 1ull);
      st[i] = 2;
      continue;
    }
    uint64_t bb = b_lo[i];
    for (int probe = 0; bb < b_hi[i] && probe < LSEL_MAX_PROBES && before(bb + 1, c_hi[i]) < K[i]; ++probe) {
      ++bb;
      c_lo[i] = c_hi[i];
      c_hi[i] = ld_u64_pol(v.dbase + bb + 1, keep);
      rv[i] = ld_v4_pol(reinterpret_cast<const uint4*>(v.dres) + bb, keep);
    }
    if (before(bb + 1, c_hi[i]) < K[i] || (int8_t)(rv[i].x & 0xFFu) == LSEL_DIR_OVER) {
      st[i] = 2;
      continue;
    }
    const uint32_t span = (uint32_t)(c_hi[i] - c_lo[i]);
    const uint32_t need_blk = (uint32_t)(K[i] - before(bb, c_lo[i]));
    const uint32_t nvalid = (uint32_t)umin64(LSEL_DIR_SB, (v.total - (bb << 13) + 511) >> 9);
    const uint4 R = rv[i];
    auto args_before = [&](uint32_t c) -> uint32_t {
      const uint32_t wsel = (c & 8) ? ((c & 4) ? R.w : R.z) : ((c & 4) ? R.y : R.x);
      const int32_t rr = (int32_t)(int8_t)(uint8_t)(wsel >> (8 * (c & 3)));
      const uint32_t t = ((span * c) >> 4) + (uint32_t)rr;
      return T_B ? t : 512u * c - t;
    };
    uint32_t si = 0;
#pragma unroll
    for (uint32_t step = 8; step; step >>= 1) {
      const uint32_t c = si + step;
      if (c < nvalid && args_before(c) < need_blk) si = c;
    }
    need[i] = need_blk - args_before(si);
    w0[i] = ((bb << 4) + si) << 3;
    const bool whole = w0[i] + 8 < v.nwords || (w0[i] + 8 == v.nwords && (v.total & 63) == 0);
    if (whole) {
      ld_v4u64_pol(v.words + w0[i], stream, wv[i][0], wv[i][1], wv[i][2], wv[i][3]);
      ld_v4u64_pol(v.words + w0[i] + 4, stream, wv[i][4], wv[i][5], wv[i][6], wv[i][7]);
      if (!T_B) {
#pragma unroll
        for (int q = 0; q < 8; ++q) wv[i][q] = ~wv[i][q];
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const uint64_t wi = w0[i] + q;
        uint64_t x = wi < v.nwords ? ld_u64_pol(v.words + wi, stream) : 0ull;
        if (!T_B) {
          x = wi < v.nwords ? ~x : 0ull;
          if (wi == v.nwords - 1 && (v.total & 63)) x &= (1ull << (v.total & 63)) - 1;
        }
        wv[i][q] = x;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    if (st[i] != 0) continue;
    uint32_t acc = __popcll(wv[i][0]), jq = 0, bq = 0;
    uint64_t wsel = wv[i][0];
#pragma unroll
    for (int q = 1; q < 8; ++q) {
      const bool past = acc < need[i];
      jq += past;
      bq = past ? acc : bq;
      wsel = past ? wv[i][q] : wsel;
      acc += __popcll(wv[i][q]);
    }
    if (acc < need[i]) {
      atomicAdd(v.misses, 1ull);
      st[i] = 2;
      continue;
    }
    res[i] = ((w0[i] + jq) << 6) + sel64(wsel, need[i] - bq) - d[i].off;
    st[i] = 1;
  }
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    const uint64_t q = q0 + (uint64_t)i * blockDim.x;
    if (q >= nq) continue;
    if (st[i] == 2) res[i] = lsel_plain(v.plain, d[i].A + k[i], d[i].off);
    out[q] = res[i];
  }
}

unsigned grid_of(uint64_t items, unsigned per_block, unsigned cap) {
  const uint64_t b = (items + per_block - 1) / per_block;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, cap));
}

int need_supports(const TreeImpl& t, uint32_t f) {
  if ((t.flags & f) != f) return fail(WTG_ERR_INVALID, "tree built without the rank/select supports this needs");
  return WTG_OK;
}

}  // namespace

int tree_level_args(TreeImpl& t, cudaStream_t s) {
  int rc;
  if (t.lvl_args_ok) return WTG_OK;
  if ((rc = need_supports(t, WTG_RANK))) return rc;
  if ((rc = t.lvl_args.ensure((t.levels + 1) * sizeof(uint64_t), s))) return rc;
  count_launch();
  level_args_kernel<<<1, 32, 0, s>>>(t.bv.rank.as<uint64_t>(), t.bits.as<uint64_t>(), t.n, t.levels,
                                     t.lvl_args.as<uint64_t>());
  WTG_CK(cudaGetLastError());
  t.lvl_args_ok = true;
  return WTG_OK;
}

int launch_level_select(TreeImpl& t, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                        uint64_t* out, cudaStream_t s) {
  int rc;
  if ((rc = need_supports(t, WTG_RANK | (t_b ? WTG_SELECT1 : WTG_SELECT0)))) return rc;
  if (nq == 0) return WTG_OK;
  if ((rc = tree_level_args(t, s))) return rc;
  const SelView v = sel_view(t.bv, t_b);
  const unsigned grid = (unsigned)((nq + 255) / 256);
  count_launch();
  if (t_b)
    level_select_kernel<1><<<grid, 256, 0, s>>>(v, t.lvl_args.as<uint64_t>(), t.n, t.levels, level, k, nq, out);
  else
    level_select_kernel<0><<<grid, 256, 0, s>>>(v, t.lvl_args.as<uint64_t>(), t.n, t.levels, level, k, nq, out);
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

LselImpl* lsel_new() { return new (std::nothrow) LselImpl(); }

namespace {

void lsel_unregister(LselImpl& m) {
  if (!m.tree) return;
  std::vector<LselImpl*>& d = m.tree->deps;
  d.erase(std::remove(d.begin(), d.end(), &m), d.end());
  m.tree = nullptr;
}

}  // namespace

TreeImpl* lsel_tree(const LselImpl& m) { return m.tree; }

void lsel_detach_all(TreeImpl& t) {
  for (LselImpl* m : t.deps) m->tree = nullptr;
  t.deps.clear();
}

void lsel_delete(LselImpl* m) {
  if (!m) return;
  // The tree (and the stream its queries ran on) may be gone: wait for the
  // whole device before handing the buffers back.
  cudaDeviceSynchronize();
  lsel_unregister(*m);
  for (int t = 0; t < 2; ++t) {
    m->lv[t].release(nullptr);
    m->rec[t].release(nullptr);
    m->plain[t].release(nullptr);
  }
  m->stats.release(nullptr);
  m->dbase.release(nullptr);
  m->dres.release(nullptr);
  cudaDeviceSynchronize();
  delete m;
}

int lsel_build(LselImpl& m, TreeImpl& t, uint32_t segments, uint32_t samples, uint32_t max_window,
               cudaStream_t s) {
  int rc;
  if (segments == 0 || samples == 0) return fail(WTG_ERR_INVALID, "segments and samples must be positive");
  if (max_window > (1u << 30)) return fail(WTG_ERR_INVALID, "max_window must be at most 2^30");
  if ((rc = need_supports(t, WTG_ALL))) return rc;
  const int L = t.levels;
  const uint64_t n = t.n;
  if (m.tree != &t) {
    lsel_unregister(m);
    t.deps.push_back(&m);
    m.tree = &t;
  }
  m.tree_gen = t.gen;
  m.segments = segments;
  m.samples = samples;
  m.max_window = max_window;
  m.L = L;
  m.n = n;
  if ((rc = tree_level_args(t, s))) return rc;
  std::vector<uint64_t> la(L + 1);
  WTG_CK(cudaMemcpyAsync(la.data(), t.lvl_args.p, (L + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));

  for (int tb = 0; tb < 2; ++tb) {
    std::vector<LselLevel>& lv = m.lv_host[tb];
    lv.assign(L, LselLevel{});
    uint64_t off = 0;
    for (int l = 0; l < L; ++l) {
      const uint64_t ones = la[l + 1] - la[l];
      LselLevel& d = lv[l];
      d.A = tb ? la[l] : (uint64_t)l * n - la[l];
      d.m = tb ? ones : n - ones;
      uint32_t g = 0;
      while (((d.m + (1ull << g) - 1) >> g) > segments) ++g;
      d.g = g;
      d.nseg = (uint32_t)((d.m + (1ull << g) - 1) >> g);
      d.rec_off = off;
      d.off = (uint64_t)l * n;
      off += d.nseg;
    }
    m.nseg[tb] = off;
    if ((rc = m.lv[tb].ensure(std::max(1, L) * sizeof(LselLevel), s))) return rc;
    if ((rc = m.rec[tb].ensure(std::max<uint64_t>(1, off) * sizeof(uint4), s))) return rc;
    WTG_CK(cudaMemcpyAsync(m.lv[tb].p, lv.data(), L * sizeof(LselLevel), cudaMemcpyHostToDevice, s));
  }
  for (int tb = 0; tb < 2; ++tb) {
    m.plain_host[tb] = sel_view(t.bv, tb);
    if ((rc = m.plain[tb].ensure(sizeof(SelView), s))) return rc;
    WTG_CK(cudaMemcpyAsync(m.plain[tb].p, &m.plain_host[tb], sizeof(SelView), cudaMemcpyHostToDevice, s));
  }
  // stats: LSEL_ST words per polarity, then the directory's overflow blocks
  if ((rc = m.stats.ensure((2 * LSEL_ST + 1) * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(m.stats.p, 0, (2 * LSEL_ST + 1) * sizeof(uint64_t), s));

  const int sms = 152;
  for (int tb = 0; tb < 2; ++tb) {
    if (!m.nseg[tb]) continue;
    count_launch();
    lsel_fit_kernel<<<grid_of(m.nseg[tb], 8, sms * 16), 256, 0, s>>>(
        sel_view(t.bv, tb), m.lv[tb].as<LselLevel>(), L, n, samples, m.nseg[tb], m.rec[tb].as<uint4>());
    WTG_CK(cudaGetLastError());
  }
  const uint64_t total = n * (uint64_t)L;
  if (total) {
    count_launch();
    lsel_bound_kernel<<<grid_of((total + 63) / 64, 256, sms * 8), 256, 0, s>>>(
        t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(), n, L, total, 1.0 / (double)n, m.lv[0].as<LselLevel>(),
        m.lv[1].as<LselLevel>(), m.rec[0].as<uint4>(), m.rec[1].as<uint4>());
    WTG_CK(cudaGetLastError());
  }
  {
    // the rank directory over the concatenated bitvector's superblocks 0..NB
    const uint64_t NB = t.bit_words >> 3;
    m.dblocks = NB / LSEL_DIR_SB + 1;  // blocks 0 .. NB / 16: every superblock with data
    if ((rc = m.dbase.ensure((m.dblocks + 1) * sizeof(uint64_t), s))) return rc;
    if ((rc = m.dres.ensure(m.dblocks * LSEL_DIR_SB, s))) return rc;
    count_launch();
    lsel_dir_kernel<<<grid_of(m.dblocks + 1, 256, 1u << 30), 256, 0, s>>>(
        t.bv.rank.as<uint64_t>(), t.bits.as<uint64_t>(), t.bit_words, m.dblocks, m.dbase.as<uint64_t>(),
        m.dres.as<int8_t>(),
        m.stats.as<unsigned long long>() + 2 * LSEL_ST);
    WTG_CK(cudaGetLastError());
  }
  for (int tb = 0; tb < 2; ++tb) {
    if (!m.nseg[tb]) continue;
    count_launch();
    lsel_stats_kernel<<<grid_of(m.nseg[tb], 256, 1u << 20), 256, 0, s>>>(
        m.rec[tb].as<uint4>(), m.nseg[tb], max_window, m.stats.as<unsigned long long>() + tb * LSEL_ST);
    WTG_CK(cudaGetLastError());
  }
  WTG_CK(cudaStreamSynchronize(s));
  return WTG_OK;
}

int lsel_info(const LselImpl& m, uint64_t info[8], cudaStream_t s) {
  uint64_t st[2 * LSEL_ST + 1];
  WTG_CK(cudaMemcpyAsync(st, m.stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  const uint64_t segs = m.nseg[0] + m.nseg[1];
  info[0] = segs;
  // the index's bytes: segment records, level records and the rank directory
  info[1] = segs * sizeof(uint4) + 2 * (uint64_t)m.L * sizeof(LselLevel) + (m.dblocks + 1) * sizeof(uint64_t) +
            m.dblocks * LSEL_DIR_SB;
  info[2] = st[0] + st[LSEL_ST + 0];
  info[3] = std::max(st[1], st[LSEL_ST + 1]);
  info[4] = st[2] + st[LSEL_ST + 2];
  info[5] = st[3] + st[LSEL_ST + 3];
  info[6] = m.segments;
  info[7] = m.samples;
  return WTG_OK;
}

int lsel_get_level(const LselImpl& m, int t_b, int level, uint64_t lvl_info[4], uint32_t* rec, uint64_t nseg,
                   cudaStream_t s) {
  if ((t_b != 0 && t_b != 1) || level < 0 || level >= m.L) return fail(WTG_ERR_INVALID, "bad level or t_b");
  const LselLevel& d = m.lv_host[t_b][level];
  lvl_info[0] = d.A;
  lvl_info[1] = d.m;
  lvl_info[2] = d.g;
  lvl_info[3] = d.nseg;
  if (rec) {
    if (nseg != d.nseg) return fail(WTG_ERR_INVALID, "nseg must equal the level's segment count");
    if (nseg) {
      WTG_CK(cudaMemcpyAsync(rec, m.rec[t_b].as<uint4>() + d.rec_off, nseg * sizeof(uint4),
                             cudaMemcpyDeviceToHost, s));
      WTG_CK(cudaStreamSynchronize(s));
    }
  }
  return WTG_OK;
}

int launch_lsel_query(LselImpl& m, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                      uint64_t* out, cudaStream_t s) {
  if (t_b != 0 && t_b != 1) return fail(WTG_ERR_INVALID, "t_b must be 0 or 1");
  if (!m.tree) return fail(WTG_ERR_INVALID, "the index's tree was freed");
  if (m.tree->gen != m.tree_gen) return fail(WTG_ERR_INVALID, "the tree was rebuilt after the index");
  if (nq == 0) return WTG_OK;
  const TreeImpl& t = *m.tree;
  LselView v;
  v.words = t.bits.as<uint64_t>();
  v.tbl = t.bv.rank.as<uint64_t>();
  v.nwords = t.bit_words;
  v.total = t.n * (uint64_t)t.levels;
  v.dbase = m.dbase.as<uint64_t>();
  v.dres = m.dres.as<int8_t>();
  v.dblocks = m.dblocks;

  v.n = t.n;
  v.L = t.levels;
  v.max_window = m.max_window;
  v.lv = m.lv[t_b].as<LselLevel>();
  v.rec = m.rec[t_b].as<uint4>();
  v.plain = m.plain[t_b].as<SelView>();
  v.misses = m.stats.as<unsigned long long>() + t_b * LSEL_ST + 3;
  constexpr int NQ = 2;  // queries per thread (1, 2, 4 measured: 2 is fastest)
  const unsigned grid = (unsigned)((nq + 256 * NQ - 1) / (256 * NQ));
  count_launch();
  if (t_b)
    lsel_query_kernel_nq<1, NQ><<<grid, 256, 0, s>>>(v, level, k, nq, out);
  else
    lsel_query_kernel_nq<0, NQ><<<grid, 256, 0, s>>>(v, level, k, nq, out);
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

}  // namespace wtg
