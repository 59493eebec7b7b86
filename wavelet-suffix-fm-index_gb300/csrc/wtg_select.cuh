// wtg_select.cuh -- device-side rank and select over the flat layouts
// (internal; shared by the query kernels and the learned select index).
#pragma once
#include "wtg_internal.cuh"

namespace wtg {

// rank_support_v<1>::rank (rank/rank_support_v_par.hpp:131-142)
__device__ __forceinline__ uint64_t rank1_dev(const uint64_t* __restrict__ tbl, const uint64_t* __restrict__ w,
                                              uint64_t idx) {
  const uint64_t* p = tbl + ((idx >> 8) & 0xFFFFFFFFFFFFFFFEull);
  uint64_t r = p[0] + ((p[1] >> (63 - 9 * ((idx & 0x1FF) >> 6))) & 0x1FF);
  if (idx & 0x3F) r += __popcll(w[idx >> 6] & ((1ull << (idx & 63)) - 1));
  return r;
}

struct SelView {
  const uint64_t* words;
  uint64_t nwords;  // data words at `words`
  const uint64_t* sb_words;
  const uint64_t* desc;
  const uint64_t* pool;
  uint64_t arg_cnt;
  uint32_t logn;
  int has_long;
  int t_b;
};

// select_support_mcl::select(i), 1 <= i <= arg_cnt
// (select/select_support_mcl_par.hpp:564-611) on the flat layout
__device__ __forceinline__ uint64_t select_dev(const SelView& v, uint64_t i) {
  if (i == 0 || i > v.arg_cnt) return NONE64;
  i = i - 1;
  const uint64_t sb = i >> 12, off = i & 0xFFF;
  const uint64_t d = v.desc[sb];
  const uint32_t wdt = (uint32_t)(d & 127);
  const uint64_t* blk = v.pool + (d >> 8);
  if (v.has_long && ((d >> 7) & 1)) return packed_get(blk, off, wdt);
  const uint64_t base = packed_get(v.sb_words, sb, v.logn);
  const uint64_t mini = packed_get(blk, off >> 6, wdt);
  if ((off & 0x3F) == 0) return base + mini;
  i = i - (sb << 12) - ((off >> 6) << 6);
  const uint64_t pos = base + mini + 1;
  uint64_t word_pos = pos >> 6;
  const uint32_t word_off = (uint32_t)(pos & 0x3F);
  if (word_pos >= v.nwords) return NONE64;
  uint64_t wd = v.words[word_pos];
  if (!v.t_b) wd = ~wd;
  const uint64_t first = wd & (~0ull << word_off);
  uint64_t args = __popcll(first);
  if (args >= i) return (word_pos << 6) + sel64(first, (uint32_t)i);
  uint64_t sum = args;
  word_pos += 1;
  if (word_pos >= v.nwords) return NONE64;
  wd = v.words[word_pos];
  if (!v.t_b) wd = ~wd;
  args = __popcll(wd);
  while (sum + args < i) {
    sum += args;
    word_pos += 1;
    if (word_pos >= v.nwords) return NONE64;  // inconsistent tables: never read past the data
    wd = v.words[word_pos];
    if (!v.t_b) wd = ~wd;
    args = __popcll(wd);
  }
  return (word_pos << 6) + sel64(wd, (uint32_t)(i - sum));
}

// Select marks of one 64-bit word wi, given K1 = ones before it: for
// select1 (x) and select0 (~x) the position of every 64th arg (low 32 bits,
// samp[dir * (arg / 64)]), every superblock start (arg 4096q) and end (arg
// 4096q + 4095).  The next multiple of 64 is d1 = (-K1) & 63 ones into the
// word, and d0 = K1 & 63 zeros into it (K0 = 64 wi - K1).  As d1 + d0 is 64
// or 0, a word holds the next 64th arg of at most one polarity unless K1 is
// a multiple of 64, and then both are the word's first one and first zero:
// one branch-free select serves every word.  zmask clears bits past the end.
// lastw1 / lastw0 become wi + 1 when the word holds a one / a zero; a caller
// that visits its words in increasing order turns the final values into
// the position after its last arg with last_arg_end().
__device__ __forceinline__ void word_marks(uint64_t x, uint32_t c, uint64_t K1, uint64_t wi, uint64_t zmask,
                                           bool sel1, bool sel0, uint32_t* __restrict__ samples, uint64_t samp_last,
                                           uint64_t* __restrict__ starts1, uint64_t* __restrict__ starts0,
                                           uint64_t* __restrict__ ends1, uint64_t* __restrict__ ends0,
                                           uint64_t& lastw1, uint64_t& lastw0) {
  const uint64_t z = ~x & zmask;
  const uint32_t cz = __popcll(z);
  const uint64_t K0 = (wi << 6) - K1;
  const uint32_t d1 = (uint32_t)(0u - (uint32_t)K1) & 63u;
  const uint32_t d0 = (uint32_t)K1 & 63u;
  const bool s1 = sel1 && d1 < c, s0 = sel0 && d0 < cz;
  if (s1 || s0) {
    const uint64_t pos = (wi << 6) + sel64_0(s1 ? x : z, s1 ? d1 : d0);
    if (s1) {
      const uint64_t k = K1 + d1;
      samples[k >> 6] = (uint32_t)pos;
      if ((k & 4095) == 0) starts1[k >> 12] = pos;
    }
    if (s0) {
      const uint64_t pos0 = s1 ? (wi << 6) + (uint64_t)(__ffsll((long long)z) - 1) : pos;
      const uint64_t k = K0 + d0;
      samples[samp_last - (k >> 6)] = (uint32_t)pos0;
      if ((k & 4095) == 0) starts0[k >> 12] = pos0;
    }
  }
  if (sel1) {
    const uint32_t e = 4095u - ((uint32_t)K1 & 4095u);
    if (e < c) ends1[(K1 + e) >> 12] = (wi << 6) + sel64_0(x, e);
    lastw1 = c ? wi + 1 : lastw1;
  }
  if (sel0) {
    const uint32_t e = 4095u - ((uint32_t)K0 & 4095u);
    if (e < cz) ends0[(K0 + e) >> 12] = (wi << 6) + sel64_0(z, e);
    lastw0 = cz ? wi + 1 : lastw0;
  }
}

// Position after the last one (t_b = 1) or zero (t_b = 0) of word lastw - 1
// of a bitvector of W words (0 when lastw is 0); read through L2
__device__ __forceinline__ uint64_t last_arg_end(const uint64_t* __restrict__ words, uint64_t lastw, uint64_t W,
                                                 uint64_t tailmask, int t_b) {
  if (!lastw) return 0;
  const uint64_t wi = lastw - 1;
  uint64_t x = __ldcg(words + wi);
  if (!t_b) x = ~x & (wi == W - 1 ? tailmask : ~0ull);
  return (wi << 6) + hi64(x) + 1;
}

inline SelView sel_view(const BvSupport& bv, int t_b) {
  const SelectDev& sd = bv.sel[t_b];
  SelView v;
  v.words = bv.words;
  v.nwords = (bv.size + 63) / 64;  // a valid query never reads past the data words
  v.sb_words = sd.sb_words.as<uint64_t>();
  v.desc = sd.desc.as<uint64_t>();
  v.pool = sd.pool.as<uint64_t>();
  v.arg_cnt = sd.arg_cnt;
  v.logn = (uint32_t)sd.logn;
  v.has_long = (int)sd.has_long;
  v.t_b = t_b;
  return v;
}

}  // namespace wtg
