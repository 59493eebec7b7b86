// wtg_bitvec.cu -- rank_support_v<1> and select_support_mcl<1>/<0>
// construction over one bitvector, on the GPU.
//
// One pass over the bitvector (bv_pass_kernel) reads each 512-bit superblock
// once and produces, through a single decoupled look-back scan of the
// superblock one-counts:
//   * the rank_support_v table (rank/rank_support_v_par.hpp:69-123): the
//     absolute count before each superblock (the exclusive scan of :112-113)
//     and the seven 9-bit in-superblock counts (:95-110), including the
//     reference's final-superblock rule (:99-108, and the (total, 0) pair when
//     the capacity is a multiple of 512);
//   * for select_support_mcl, the position of every 64th arg (its
//     superblock starts are every 64th of those) and of every arg that ends a
//     superblock (select_support_mcl_par.hpp:492-523);
// The select structure is then finished per superblock: the long/mini choice
// (span > log^4 n) and widths (:525-543), the pool offsets (a scan), the mini
// blocks from the samples (init_miniblock_serial :440-481), the long blocks by
// re-reading their span (init_longblock_serial :401-438) and m_superblock
// (:546-549).
#include <algorithm>
#include <mutex>

#include "wtg_internal.cuh"
#include "wtg_select.cuh"

namespace wtg {

WTG_WAIT_LIMIT_SETTER(bitvec)

constexpr int BV_THREADS = 256;  // one 512-bit superblock per thread

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  return v;
}

// One pass over the bitvector: lane per 64-bit word, 8 lanes per 512-bit
// superblock, a tile of 256 superblocks per CTA (coalesced 2 KB rows), one
// decoupled look-back scan of the tile one-counts.
constexpr int BVT_ITER = 8;                        // rows of 256 words per tile
constexpr int BVT_SB = BVT_ITER * BV_THREADS / 8;  // superblocks per tile

__global__ void __launch_bounds__(BV_THREADS)
    bv_pass_kernel(const uint64_t* __restrict__ words, uint64_t size, uint64_t W, uint64_t NB, uint32_t flags,
                   uint64_t* __restrict__ rank, uint32_t* __restrict__ samples, uint64_t samp_last,
                   uint64_t* __restrict__ starts1, uint64_t* __restrict__ starts0, uint64_t* __restrict__ ends1,
                   uint64_t* __restrict__ ends0, unsigned long long* info, uint64_t* status, uint32_t* counter,
                   uint32_t* err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_sb[BVT_SB];
  __shared__ uint64_t s_prefix;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  if (tile >= gridDim.x) return;  // only when the counter did not start at 0 (a stalled pass)
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g8 = lane & 7;
  const uint64_t wbase = (uint64_t)tile * (BVT_ITER * BV_THREADS);
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  uint64_t w[BVT_ITER];
  uint32_t c[BVT_ITER], inc[BVT_ITER];
#pragma unroll
  for (int j = 0; j < BVT_ITER; ++j) {
    const uint64_t wi = wbase + j * BV_THREADS + tid;
    uint64_t x = wi < W ? __ldg(&words[wi]) : 0ull;
    if (wi == W - 1) x &= tailmask;
    w[j] = x;
    c[j] = __popcll(x);
    uint32_t v = c[j];
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {  // inclusive scan within the superblock's 8 lanes
      const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
      if (g8 >= (uint32_t)o) v += t;
    }
    inc[j] = v;
    if (g8 == 7) s_sb[j * (BV_THREADS / 8) + warp * 4 + (lane >> 3)] = v;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int PER = BVT_SB / 32;
    uint32_t loc[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      loc[q] = s_sb[lane * PER + q];
      sum += loc[q];
    }
    uint32_t incw = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incw, o);
      if (lane >= (uint32_t)o) incw += t;
    }
    uint32_t run = incw - sum;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      s_sb[lane * PER + q] = run;
      run += loc[q];
    }
    const uint64_t total = __shfl_sync(0xffffffffu, incw, 31);
    uint64_t prefix = 0;
    if (tile == 0) {
      if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, total);
    } else {
      if (lane == 0) lb_publish(status, tile, LB_FLAG_AGG, total);
      prefix = lb_lookback_warp(status, tile, err);
      if (lane == 0) lb_publish(status, tile, LB_FLAG_INC, prefix + total);
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  const uint64_t tprefix = s_prefix;
  const uint64_t r_last = W - 8 * NB;  // words of the final superblock
  uint64_t last1 = 0, last0 = 0;
#pragma unroll
  for (int j = 0; j < BVT_ITER; ++j) {
    const uint32_t sbl = j * (BV_THREADS / 8) + warp * 4 + (lane >> 3);
    const uint64_t b = (uint64_t)tile * BVT_SB + sbl;  // superblock
    const uint64_t wi = wbase + j * BV_THREADS + tid;
    const uint64_t sb_before = tprefix + s_sb[sbl];    // ones before the superblock
    const uint32_t excl = inc[j] - c[j];               // ones before the word in its superblock
    const uint32_t sbt = __shfl_sync(0xffffffffu, inc[j], (lane & ~7u) + 7);  // ones in the superblock
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
      info[INF_M1] = sb_before + sbt;
      info[INF_M0] = size - (sb_before + sbt);
    }
    if (wi < W)
      word_marks(w[j], c[j], sb_before + excl, wi, wi == W - 1 ? tailmask : ~0ull, flags & WTG_SELECT1,
                 flags & WTG_SELECT0, samples, samp_last, starts1, starts0, ends1, ends0, last1, last0);
  }
  last1 = warp_max_u64(last_arg_end(words, last1, W, tailmask, 1));
  last0 = warp_max_u64(last_arg_end(words, last0, W, tailmask, 0));
  if (lane == 0) {
    if (last1) atomicMax(&info[INF_LAST1], (unsigned long long)last1);
    if (last0) atomicMax(&info[INF_LAST0], (unsigned long long)last0);
  }
}

// position after the last one (t_b = 1) or zero (t_b = 0) of superblock sb
// (eight words, all inside the bitvector); read through L2
__device__ __forceinline__ uint64_t last_arg_end_sb(const uint64_t* __restrict__ words, uint64_t sb, int t_b) {
  for (int j = 7; j >= 0; --j) {
    uint64_t x = __ldcg(words + 8 * sb + j);
    if (!t_b) x = ~x;
    if (x) return ((8 * sb + j) << 6) + hi64(x) + 1;
  }
  return 0;
}

// Rank table and select samples of a wavelet tree's concatenated bitvector
// when n % 512 == 0: superblock b is chunk c of level l (b = l * n/512 + c),
// and the zeros before it are the zeros of the levels before l (lvl_zb) plus
// the chunk's prefix within its level (the level passes' chunk counts,
// scanned) -- no scan over the bits.  Levels l0..l1-1; thread per
// superblock, grid-stride over each level's superblocks.
//
// Per word, the work is one in-word select at most (the next 64th one or
// zero, see word_marks) in 32-bit arithmetic on per-superblock 64-bit bases:
// the select1 samples of a superblock are consecutive from index
// ceil(ones before / 64), the select0 samples consecutive (descending from
// the back) from ceil(zeros before / 64).  The last two steps of the select
// read a 256 x 8 table of in-byte selects from shared memory.  A superblock
// holds at most one superblock end per polarity (512 < 4096 args), resolved
// once per superblock; the last word holding a one / a zero is resolved once
// per thread from the last such superblock.
__global__ void __launch_bounds__(256)
    rs_levels_kernel(const uint64_t* __restrict__ words, int l0, int l1, uint64_t chunks_per_level,
                     const uint32_t* __restrict__ chunkpre, uint64_t prestride, const uint64_t* __restrict__ lvl_zb,
                     uint32_t flags, uint64_t* __restrict__ rank, uint32_t* __restrict__ samples, uint64_t samp_last,
                     uint64_t* __restrict__ starts1, uint64_t* __restrict__ starts0, uint64_t* __restrict__ ends1,
                     uint64_t* __restrict__ ends0, unsigned long long* info) {
  __shared__ uint8_t lut[256 * 8];  // lut[byte * 8 + r] = position of the r-th set bit of byte
  sel_lut_init(lut);
  __syncthreads();
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  const bool sel1 = flags & WTG_SELECT1, sel0 = flags & WTG_SELECT0, sel = sel1 || sel0;
  uint64_t last_sb1 = ~0ull, last_sb0 = ~0ull;  // last superblocks holding a one / a zero
  // thread per 512-bit superblock: its eight words in four 16-byte loads,
  // counts and fields in registers, one 16-byte rank entry
  for (int l = l0; l < l1; ++l) {
    const uint64_t zl = lvl_zb[l];
    const uint32_t* __restrict__ pre = chunkpre + (uint64_t)l * prestride;
    for (uint64_t c = tid; c < chunks_per_level; c += nthreads) {
      const uint64_t b = (uint64_t)l * chunks_per_level + c;  // superblock
      const ulonglong2* p = reinterpret_cast<const ulonglong2*>(words + 8 * b);
      const ulonglong2 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3);
      const uint64_t w[8] = {q0.x, q0.y, q1.x, q1.y, q2.x, q2.y, q3.x, q3.y};
      const uint64_t zb = zl + __ldg(pre + c);  // zeros before the superblock
      const uint64_t sb_before = 512 * b - zb;  // ones before the superblock
      const uint32_t pos_base = (uint32_t)(512 * b);
      const uint32_t k1_base = (uint32_t)sb_before, k0_base = (uint32_t)zb;
      // next samples of this superblock: select1 from the front, select0 from the back
      uint32_t* __restrict__ p1 = samples + ((sb_before + 63) >> 6);
      uint32_t* __restrict__ p0 = samples + (samp_last - ((zb + 63) >> 6));
      uint32_t excl = 0;  // ones before the word within the superblock
      uint32_t n1 = 0, n0 = 0;
      uint64_t part = 0;
      uint32_t cnt[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint64_t x = w[j];
        const uint32_t cl = __popc((uint32_t)x);
        const uint32_t cj = cl + __popc((uint32_t)(x >> 32));
        cnt[j] = cj;
        if (j) part |= (uint64_t)excl << (63 - 9 * j);
        if (sel) {
          // branch-free: the select runs for every word, the stores are predicated
          const uint32_t K1 = k1_base + excl;            // ones before the word (mod 2^32)
          const uint32_t K0 = k0_base + 64u * j - excl;  // zeros before it
          const uint32_t d1 = (0u - K1) & 63u, d0 = K1 & 63u;
          const bool s1 = sel1 && d1 < cj, s0 = sel0 && d0 < 64u - cj;
          const uint32_t off = sel64_lut(s1 ? x : ~x, s1 ? d1 : d0, s1 ? cl : 32u - cl, lut);
          // both polarities only when K1 % 64 == 0: the word's first one and first zero
          const uint32_t off0 = s1 ? (uint32_t)(__ffsll((long long)~x) - 1) : off;
          const uint32_t pos = pos_base + 64u * j;
          if (s1) p1[n1] = pos + off;
          if (s0) *(p0 - n0) = pos + off0;
          if (s1 && ((K1 + d1) & 4095u) == 0) starts1[(sb_before + excl + d1) >> 12] = 512 * b + 64 * j + off;
          if (s0 && ((K0 + d0) & 4095u) == 0)
            starts0[(zb + 64 * j - excl + d0) >> 12] = 512 * b + 64 * j + off0;
          n1 += s1;
          n0 += s0;
        }
        excl += cj;
      }
      if (flags & WTG_RANK) reinterpret_cast<ulonglong2*>(rank)[b] = make_ulonglong2(sb_before, part);
      if (sel) {
        // superblock ends: arg 4095 of a 4096-arg superblock, at most one per
        // polarity in 512 bits; one scan serves the lane's first polarity,
        // the rare superblock that ends one of each takes a second
        const uint32_t cz = 512u - excl;
        const uint32_t e1 = 4095u - (k1_base & 4095u), e0 = 4095u - (k0_base & 4095u);
        bool h1 = sel1 && e1 < excl, h0 = sel0 && e0 < cz;
        // the lanes still inside the superblock loop (its last round may hold fewer)
        const uint32_t live = __activemask();
        while (__any_sync(live, h1 || h0)) {
          const bool t1 = h1;  // this round's polarity
          const uint32_t e = t1 ? e1 : e0;
          uint32_t before = 0, r = 0;
          uint64_t xx = 0, jj = 0;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const uint32_t cj = t1 ? cnt[j] : 64u - cnt[j];
            const bool here = before <= e && e < before + cj;
            xx = here ? w[j] : xx;
            r = here ? e - before : r;
            jj = here ? (uint64_t)j : jj;
            before += cj;
          }
          xx = t1 ? xx : ~xx;
          const uint64_t pos = 512 * b + 64 * jj + sel64_lut(xx, r, __popc((uint32_t)xx), lut);
          if (h1) ends1[(sb_before + e1) >> 12] = pos;
          else if (h0) ends0[(zb + e0) >> 12] = pos;
          if (h1) h1 = false;
          else h0 = false;
        }
        last_sb1 = excl ? b : last_sb1;
        last_sb0 = cz ? b : last_sb0;
      }
    }
  }
  if (sel) {
    const uint64_t last1 = warp_max_u64(last_sb1 == ~0ull ? 0 : last_arg_end_sb(words, last_sb1, 1));
    const uint64_t last0 = warp_max_u64(last_sb0 == ~0ull ? 0 : last_arg_end_sb(words, last_sb0, 0));
    if ((threadIdx.x & 31) == 0) {
      if (last1) atomicMax(&info[INF_LAST1], (unsigned long long)last1);
      if (last0) atomicMax(&info[INF_LAST0], (unsigned long long)last0);
    }
  }
}

// arg counts and the rank pair after the last superblock, (total, 0)
// (rank_support_v_par.hpp:95-110 with capacity % 512 == 0)
__global__ void rs_levels_totals_kernel(const uint64_t* lvl_zb, int L, uint64_t size, uint64_t NB, uint64_t* rank,
                                        unsigned long long* info) {
  const uint64_t z = lvl_zb[L];
  info[INF_M1] = size - z;
  info[INF_M0] = z;
  if (rank) {
    rank[2 * NB] = size - z;
    rank[2 * NB + 1] = 0;
  }
}

// zeros before levels l0+1..l1: lvl_zb[l + 1] = lvl_zb[l] + zeros of level l,
// from lvl_zb[l0] (0 for l0 == 0)
__global__ void level_zeros_kernel(const uint32_t* __restrict__ chunkcnt, const uint32_t* __restrict__ chunkpre,
                                   uint64_t stride, uint64_t nchunks, int l0, int l1, uint64_t* __restrict__ lvl_zb) {
  if (l0 == 0) lvl_zb[0] = 0;
  uint64_t acc = lvl_zb[l0];
  for (int l = l0; l < l1; ++l) {
    acc += (uint64_t)chunkpre[l * stride + nchunks - 1] + chunkcnt[l * stride + nchunks - 1];
    lvl_zb[l + 1] = acc;
  }
}

int bv_levels_begin(BvSupport& bv, const uint64_t* d_words, uint64_t n, int L, uint32_t flags, cudaStream_t s) {
  return bv_prepare(bv, d_words, n * (uint64_t)L, flags, s);
}

int bv_levels_pass(BvSupport& bv, uint64_t n, int l0, int l1, const uint32_t* chunkcnt, const uint32_t* chunkpre,
                   uint64_t stride, uint64_t nchunks, uint64_t* lvl_zb, cudaStream_t s) {
  if (l1 <= l0) return WTG_OK;
  const uint64_t samp_n = bv.size / 64 + 2;
  level_zeros_kernel<<<1, 1, 0, s>>>(chunkcnt, chunkpre, stride, nchunks, l0, l1, lvl_zb);
  count_launch();
  WTG_CK(cudaGetLastError());
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const uint64_t per_level = n / 512;  // superblocks per level, one thread each
  const unsigned grid = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>((per_level + 255) / 256, (uint64_t)sms * 8));
  prof_begin(PROF_BVPASS, s);
  rs_levels_kernel<<<grid, 256, 0, s>>>(
      bv.words, l0, l1, n / 512, chunkpre, stride, lvl_zb, bv.flags, bv.rank.as<uint64_t>(),
      bv.samples.as<uint32_t>(), samp_n - 1, bv.sel[1].starts.as<uint64_t>(), bv.sel[0].starts.as<uint64_t>(),
      bv.sel[1].ends.as<uint64_t>(), bv.sel[0].ends.as<uint64_t>(), bv.info.as<unsigned long long>());
  prof_end(PROF_BVPASS, s);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int bv_levels_end(BvSupport& bv, int L, const uint64_t* lvl_zb, uint32_t* d_err, cudaStream_t s) {
  const uint64_t NB = bv.size / 512;
  rs_levels_totals_kernel<<<1, 1, 0, s>>>(lvl_zb, L, bv.size, NB,
                                         (bv.flags & WTG_RANK) ? bv.rank.as<uint64_t>() : nullptr,
                                         bv.info.as<unsigned long long>());
  count_launch();
  WTG_CK(cudaGetLastError());
  if (bv.rank_done) WTG_CK(cudaEventRecord(bv.rank_done, s));
  return bv_finish(bv, d_err, s);
}

// per superblock: long/mini choice, width and pool words
__global__ void select_desc_kernel(int t_b, const uint64_t* __restrict__ starts,
                                   const uint64_t* __restrict__ ends, unsigned long long* info, uint64_t logn4,
                                   uint64_t nsb_cap, uint64_t* __restrict__ descw, uint64_t* __restrict__ sizes,
                                   uint64_t* __restrict__ long_list) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsb_cap) return;
  const uint64_t m = info[t_b ? INF_M1 : INF_M0];
  const uint64_t nsb = (m + 4095) >> 12;
  if (i >= nsb) {
    sizes[i] = 0;
    return;
  }
  const uint64_t start = starts[i];
  const uint64_t end = (i + 1 < nsb) ? ends[i] : (uint64_t)info[t_b ? INF_LAST1 : INF_LAST0] - 1;
  const uint64_t span = end - start;
  const uint64_t lng = span > logn4;
  const uint64_t wdt = lng ? hi64(end) + 1 : hi64(span) + 1;
  descw[i] = (lng << 7) | wdt;
  sizes[i] = lng ? 64 * wdt : wdt;
  if (lng) {
    unsigned long long slot = atomicAdd(&info[t_b ? INF_NLONG1 : INF_NLONG0], 1ull);
    long_list[slot] = i;
  }
}

__global__ void select_pool_total_kernel(int t_b, unsigned long long* info, const uint64_t* sizes,
                                         const uint64_t* offs) {
  const uint64_t m = info[t_b ? INF_M1 : INF_M0];
  const uint64_t nsb = (m + 4095) >> 12;
  info[t_b ? INF_POOL1 : INF_POOL0] = nsb ? offs[nsb - 1] + sizes[nsb - 1] : 0;
}

// Two superblocks per warp (lanes 0-15 pack superblock 2w's words, lanes
// 16-31 superblock 2w+1's): final descriptors and the 64-entry mini blocks.
// A mini block's words are few (its width, at most 32), so one superblock per
// warp left half of the lanes idle while the others packed.
__global__ void __launch_bounds__(256)
    select_mini_kernel(int t_b, uint64_t nsb, uint64_t m, const uint32_t* __restrict__ samples, uint64_t samp_last,
                       const uint64_t* __restrict__ descw, const uint64_t* __restrict__ offs,
                       uint64_t* __restrict__ desc, uint64_t* __restrict__ pool) {
  __shared__ uint64_t ent[256 / 32][2][64];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t i0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2;
  if (i0 >= nsb) return;
  auto samp = [&](uint64_t k) { return t_b ? samples[k] : samples[samp_last - k]; };
  // positions are kept mod 2^32; a mini block spans at most log^4 n < 2^32
  // bits, so the offsets are exact
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint64_t i = i0 + h;
    if (i < nsb) {  // warp-uniform
      const uint32_t start = samp(64 * i);
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const uint32_t j = lane + 32 * g;
        const uint64_t k = 4096 * i + 64 * (uint64_t)j;
        ent[warp][h][j] = (k < m) ? (uint64_t)(uint32_t)(samp(64 * i + j) - start) : 0;
      }
    }
  }
  __syncwarp();
  const uint32_t h = lane >> 4, ql = lane & 15;
  const uint64_t i = i0 + h;
  if (i >= nsb) return;
  const uint64_t d = descw[i];
  const uint64_t off = offs[i];
  if (ql == 0) desc[i] = (off << 8) | (d & 255);
  if ((d >> 7) & 1) return;  // long block
  const uint32_t wdt = (uint32_t)(d & 127);
  // entry indices of a word's first and last bit: floor(x / wdt) for
  // x < 2^11 by one multiply with ceil(2^26 / wdt) (exact for x < 2^20,
  // wdt <= 64), not two divisions per word
  const uint64_t rcp = ((1ull << 26) + wdt - 1) / wdt;
  for (uint32_t q = ql; q < wdt; q += 16) {
    const uint32_t lo = q * 64;
    const uint32_t j0 = (uint32_t)(((uint64_t)lo * rcp) >> 26), j1 = (uint32_t)(((uint64_t)(lo + 63) * rcp) >> 26);
    uint64_t out = 0;
    for (uint32_t j = j0; j <= j1 && j < 64; ++j) {
      const uint64_t v = ent[warp][h][j];  // < 2^wdt
      const int32_t sh = (int32_t)(j * wdt) - (int32_t)lo;
      out |= sh >= 0 ? (v << sh) : (v >> (-sh));
    }
    pool[off + q] = out;
  }
}

// m_superblock: entry i = position of arg 4096*i, width logn
__global__ void select_sb_pack_kernel(uint64_t nsb, uint32_t logn, const uint64_t* __restrict__ starts,
                                      uint64_t nwords, uint64_t* __restrict__ sb_words) {
  uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nwords) return;
  sb_words[q] = packed_word(q, logn, nsb, [&](uint64_t i) { return starts[i]; });
}

// Long blocks, step 1: the position of every arg of every long superblock,
// one thread per entry (init_longblock_serial, :401-438, restated).  Long
// superblocks are where args are sparse, so instead of scanning their span the
// k-th arg is located by binary search over the rank table's absolute counts
// (between the two samples that bracket it), then within its 512-bit
// superblock by popcounts of at most 8 words.
__device__ __forceinline__ uint64_t args_before_sb(int t_b, const uint64_t* __restrict__ rank, uint64_t b) {
  const uint64_t r = rank[2 * b];
  return t_b ? r : 512 * b - r;
}

__global__ void __launch_bounds__(256)
    select_long_fill_kernel(int t_b, const uint64_t* __restrict__ words, uint64_t size, uint64_t W,
                            const uint64_t* __restrict__ rank, const uint64_t* __restrict__ starts,
                            const uint64_t* __restrict__ ends, const unsigned long long* info,
                            const uint64_t* __restrict__ long_list, uint64_t* __restrict__ ent, uint32_t* err) {
  const uint64_t gt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t m = info[t_b ? INF_M1 : INF_M0];
  const uint64_t last = info[t_b ? INF_LAST1 : INF_LAST0];  // last arg position + 1
  const uint64_t nlong = info[t_b ? INF_NLONG1 : INF_NLONG0];
  const uint64_t li = gt >> 12, j = gt & 4095;
  if (li >= nlong) return;
  const uint64_t i = long_list[li];
  const uint64_t k = 4096 * i + j;  // 0-based arg index
  if (k >= m) return;               // entries past the arg count stay zero
  const uint64_t nsb = (m + 4095) >> 12;
  const uint64_t plo = starts[i];
  const uint64_t phi = i + 1 < nsb ? ends[i] : last - 1;
  uint64_t lo = plo >> 9, hi = phi >> 9;  // largest b in [lo, hi] with args_before_sb(b) <= k
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) >> 1;
    if (args_before_sb(t_b, rank, mid) <= k) lo = mid;
    else hi = mid - 1;
  }
  uint64_t rem = k - args_before_sb(t_b, rank, lo);
  const uint64_t tailmask = (size & 63) ? ((1ull << (size & 63)) - 1) : ~0ull;
  for (uint64_t wi = 8 * lo; wi < 8 * lo + 8 && wi < W; ++wi) {
    uint64_t x = words[wi];
    if (!t_b) x = ~x;
    if (wi == W - 1) x &= tailmask;
    const uint32_t c = __popcll(x);
    if (rem < c) {
      ent[(li << 12) + j] = (wi << 6) + sel64(x, (uint32_t)rem + 1);
      return;
    }
    rem -= c;
  }
  atomicCAS(err, 0u, (uint32_t)DERR_SELECT_OVERFLOW);  // tables inconsistent
}

// Long blocks, step 2: pack each long block's 4096 positions (width hi(end)+1).
__global__ void __launch_bounds__(256)
    select_long_pack_kernel(int t_b, const unsigned long long* info, const uint64_t* __restrict__ long_list,
                            const uint64_t* __restrict__ descw, const uint64_t* __restrict__ offs,
                            const uint64_t* __restrict__ ent, uint64_t* __restrict__ pool) {
  const uint64_t nlong = info[t_b ? INF_NLONG1 : INF_NLONG0];
  for (uint64_t li = blockIdx.x; li < nlong; li += gridDim.x) {
    const uint64_t i = long_list[li];
    const uint32_t wdt = (uint32_t)(descw[i] & 127);
    const uint64_t off = offs[i];
    const uint64_t* e = ent + li * 4096;
    for (uint64_t q = threadIdx.x; q < 64ull * wdt; q += blockDim.x)
      pool[off + q] = packed_word(q, wdt, 4096, [&](uint64_t j) { return e[j]; });
  }
}

// ------------------------------------------------------------------ host

static uint32_t logn_of(uint64_t size) {
  uint64_t cap = (size + 63) / 64 * 64;
  return hi64(cap) + 1;
}

void bv_release(BvSupport& bv, cudaStream_t s) {
  bv.rank.release(s);
  bv.samples.release(s);
  bv.info.release(s);
  bv.status.release(s);
  bv.scan_tmp.release(s);
  for (auto& sd : bv.sel) {
    sd.ends.release(s);
    sd.desc.release(s);
    sd.sizes.release(s);
    sd.sb_words.release(s);
    sd.pool.release(s);
    sd.long_list.release(s);
    sd.long_ent.release(s);
    sd.starts.release(s);
  }
}

int bv_prepare(BvSupport& bv, const uint64_t* d_words, uint64_t size, uint32_t& flags, cudaStream_t s) {
  int rc;
  // select's long blocks are filled through the rank table, so it is built
  // whenever a select support is
  if (flags & (WTG_SELECT1 | WTG_SELECT0)) flags |= WTG_RANK;
  bv.size = size;
  bv.words = d_words;
  bv.flags = flags;
  const uint64_t W = (size + 63) / 64;
  const uint64_t NB = W >> 3;
  const uint64_t nsb_cap = size / 4096 + 2;
  const uint64_t samp_n = W + 2;
  if ((rc = bv.info.ensure(INF_N * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(bv.info.p, 0, INF_N * sizeof(uint64_t), s));
  if (flags & WTG_RANK)
    if ((rc = bv.rank.ensure(2 * (NB + 1) * sizeof(uint64_t), s))) return rc;
  if (flags & (WTG_SELECT1 | WTG_SELECT0))
    if ((rc = bv.samples.ensure(samp_n * sizeof(uint32_t), s))) return rc;
  for (int t_b = 0; t_b < 2; ++t_b) {
    if (!(flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) continue;
    SelectDev& sd = bv.sel[t_b];
    if ((rc = sd.ends.ensure(nsb_cap * sizeof(uint64_t), s))) return rc;
    if ((rc = sd.starts.ensure(nsb_cap * sizeof(uint64_t), s))) return rc;
    if ((rc = sd.desc.ensure(2 * nsb_cap * sizeof(uint64_t), s))) return rc;   // [final | working]
    if ((rc = sd.sizes.ensure(2 * nsb_cap * sizeof(uint64_t), s))) return rc;  // [sizes | offsets]
    if ((rc = sd.long_list.ensure(nsb_cap * sizeof(uint64_t), s))) return rc;
  }
  return WTG_OK;
}

int bv_pass(BvSupport& bv, uint32_t* d_err, cudaStream_t s) {
  int rc;
  const uint64_t size = bv.size;
  const uint64_t W = (size + 63) / 64;
  const uint64_t NB = W >> 3;
  const uint64_t samp_n = W + 2;
  const uint64_t tiles = (NB + 1 + BVT_SB - 1) / BVT_SB;
  if (tiles > 0x7fffffffull) return fail(WTG_ERR_INVALID, "bitvector too large");
  if ((rc = bv.status.ensure((tiles + 1) * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(bv.status.p, 0, (tiles + 1) * sizeof(uint64_t), s));
  if (test_take_lookback_stall()) {  // tile 0 is never taken: every look-back wait on it runs out
    static const uint32_t one = 1;
    WTG_CK(cudaMemcpyAsync(bv.status.p, &one, sizeof(one), cudaMemcpyHostToDevice, s));
  }
  prof_begin(PROF_BVPASS, s);
  bv_pass_kernel<<<(unsigned)tiles, BV_THREADS, 0, s>>>(
      bv.words, size, W, NB, bv.flags, bv.rank.as<uint64_t>(), bv.samples.as<uint32_t>(), samp_n - 1,
      bv.sel[1].starts.as<uint64_t>(), bv.sel[0].starts.as<uint64_t>(), bv.sel[1].ends.as<uint64_t>(),
      bv.sel[0].ends.as<uint64_t>(), bv.info.as<unsigned long long>(), bv.status.as<uint64_t>() + 1,
      bv.status.as<uint32_t>(), d_err);
  prof_end(PROF_BVPASS, s);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int bv_finish(BvSupport& bv, uint32_t* d_err, cudaStream_t s) {
  int rc;
  const uint32_t flags = bv.flags;
  if (!(flags & (WTG_SELECT1 | WTG_SELECT0))) return WTG_OK;
  const uint64_t size = bv.size;
  const uint64_t W = (size + 63) / 64;
  const uint64_t nsb_cap = size / 4096 + 2;
  const uint64_t samp_n = W + 2;
  const uint32_t logn = logn_of(size);
  const uint64_t logn4 = (uint64_t)(uint32_t)(logn * logn * logn * logn);  // uint32 as in initData
  const uint64_t* d_words = bv.words;
  unsigned long long* info = bv.info.as<unsigned long long>();
  uint32_t* samples = bv.samples.as<uint32_t>();

  for (int t_b = 0; t_b < 2; ++t_b) {
    if (!(flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) continue;
    SelectDev& sd = bv.sel[t_b];
    uint64_t* descw = sd.desc.as<uint64_t>() + nsb_cap;
    uint64_t* sizes = sd.sizes.as<uint64_t>();
    uint64_t* offs = sizes + nsb_cap;
    prof_begin(PROF_SELECT, s);
    select_desc_kernel<<<(unsigned)((nsb_cap + 255) / 256), 256, 0, s>>>(
        t_b, sd.starts.as<uint64_t>(), sd.ends.as<uint64_t>(), info, logn4, nsb_cap, descw, sizes,
        sd.long_list.as<uint64_t>());
    prof_end(PROF_SELECT, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    if ((rc = scan_exclusive_u64(sizes, offs, nsb_cap, bv.scan_tmp, d_err, s))) return rc;
    prof_begin(PROF_SELECT, s);
    select_pool_total_kernel<<<1, 1, 0, s>>>(t_b, info, sizes, offs);
    prof_end(PROF_SELECT, s);
    count_launch();
    WTG_CK(cudaGetLastError());
  }

  // the pool sizes decide the allocations: one small read-back
  uint64_t h[INF_N];
  WTG_CK(cudaMemcpyAsync(h, info, sizeof(h), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));

  for (int t_b = 0; t_b < 2; ++t_b) {
    if (!(flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) continue;
    SelectDev& sd = bv.sel[t_b];
    const uint64_t m = h[t_b ? INF_M1 : INF_M0];
    sd.arg_cnt = m;
    sd.logn = logn;
    sd.logn4 = logn4;
    sd.nsb = (m + 4095) >> 12;
    sd.has_long = h[t_b ? INF_NLONG1 : INF_NLONG0] ? 1 : 0;
    sd.pool_nwords = h[t_b ? INF_POOL1 : INF_POOL0];
    sd.sb_nwords = (sd.nsb * logn + 63) / 64;
    if ((rc = sd.pool.ensure((sd.pool_nwords + 1) * sizeof(uint64_t), s))) return rc;
    if ((rc = sd.sb_words.ensure((sd.sb_nwords + 1) * sizeof(uint64_t), s))) return rc;
    if (sd.nsb == 0) continue;
    uint64_t* descw = sd.desc.as<uint64_t>() + nsb_cap;
    uint64_t* offs = sd.sizes.as<uint64_t>() + nsb_cap;
    prof_begin(PROF_SELECT, s);
    select_mini_kernel<<<(unsigned)(((sd.nsb + 1) / 2 * 32 + 255) / 256), 256, 0, s>>>(
        t_b, sd.nsb, m, samples, samp_n - 1, descw, offs, sd.desc.as<uint64_t>(), sd.pool.as<uint64_t>());
    prof_end(PROF_SELECT, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    prof_begin(PROF_SELECT, s);
    select_sb_pack_kernel<<<(unsigned)((sd.sb_nwords + 255) / 256), 256, 0, s>>>(
        sd.nsb, logn, sd.starts.as<uint64_t>(), sd.sb_nwords, sd.sb_words.as<uint64_t>());
    prof_end(PROF_SELECT, s);
    count_launch();
    WTG_CK(cudaGetLastError());
    const uint64_t nlong = h[t_b ? INF_NLONG1 : INF_NLONG0];
    if (nlong) {
      if ((rc = sd.long_ent.ensure(nlong * 4096 * sizeof(uint64_t), s))) return rc;
      WTG_CK(cudaMemsetAsync(sd.long_ent.p, 0, nlong * 4096 * sizeof(uint64_t), s));
      prof_begin(PROF_SELECT, s);
      select_long_fill_kernel<<<(unsigned)((nlong * 4096 + 255) / 256), 256, 0, s>>>(
          t_b, d_words, size, W, bv.rank.as<uint64_t>(), sd.starts.as<uint64_t>(), sd.ends.as<uint64_t>(), info,
          sd.long_list.as<uint64_t>(), sd.long_ent.as<uint64_t>(), d_err);
      prof_end(PROF_SELECT, s);
      count_launch();
      WTG_CK(cudaGetLastError());
      unsigned grid = (unsigned)std::min<uint64_t>(nlong, 8 * 152);
      prof_begin(PROF_SELECT, s);
      select_long_pack_kernel<<<grid, 256, 0, s>>>(t_b, info, sd.long_list.as<uint64_t>(), descw, offs,
                                                   sd.long_ent.as<uint64_t>(), sd.pool.as<uint64_t>());
      prof_end(PROF_SELECT, s);
      count_launch();
      WTG_CK(cudaGetLastError());
    }
  }
  return WTG_OK;
}

int bv_build(BvSupport& bv, const uint64_t* d_words, uint64_t size, uint32_t flags, uint32_t* d_err,
             cudaStream_t s) {
  int rc;
  if ((rc = bv_prepare(bv, d_words, size, flags, s))) return rc;
  if ((rc = bv_pass(bv, d_err, s))) return rc;
  if (bv.rank_done) WTG_CK(cudaEventRecord(bv.rank_done, s));
  return bv_finish(bv, d_err, s);
}

// ------------------------------------------------ allocation-free rank build
//
// For callers that must not allocate device memory themselves or through
// this library: code running where the allocator is off limits (inside a
// memory budget owned by another framework, during a phase where cudaMalloc
// would synchronise the device, or on a pool that forbids new allocations).
// The rank pass needs scratch for its look-back status words, its tile
// counter and a few device scalars; here they live in one file-scope device
// array of fixed size, so the call allocates nothing.  Every GPU that loads
// the library holds this array until the process exits.
constexpr uint64_t NOALLOC_MAX_BITS = 1ull << 34;  // 16 Gbit (2 GiB of bits)
constexpr uint64_t NOALLOC_TILES = ((NOALLOC_MAX_BITS >> 9) + 1 + BVT_SB - 1) / BVT_SB;
constexpr uint64_t NOALLOC_WORDS = 1 + NOALLOC_TILES + INF_N + 1;  // counter, status, info, error
static __device__ __align__(256) uint64_t g_noalloc_scratch[NOALLOC_WORDS];

static uint64_t* noalloc_scratch_ptr(int dev, int* rc) {
  static std::mutex mu;
  static uint64_t* ptrs[64] = {nullptr};
  if (dev < 0 || dev >= 64) {
    *rc = fail(WTG_ERR_CUDA, "device ordinal out of range");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  // set-up, once per device, with that device current.  The address is kept
  // for the life of the process, so it is not valid after a cudaDeviceReset.
  if (!ptrs[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *rc = cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
      return nullptr;
    }
    ptrs[dev] = (uint64_t*)p;
  }
  *rc = WTG_OK;
  return ptrs[dev];
}

}  // namespace wtg

extern "C" int wtg_rank_build_noalloc(const uint64_t* d_words, uint64_t size_bits, uint64_t* d_rank,
                                      void* stream) {
  using namespace wtg;
  if ((!d_words && size_bits) || !d_rank) return fail(WTG_ERR_INVALID, "null argument");
  if (size_bits > NOALLOC_MAX_BITS)
    return fail(WTG_ERR_RANGE, "wtg_rank_build_noalloc: size_bits exceeds its fixed scratch (at most 2^34 bits)");
  int dev = 0;
  WTG_CK(cudaGetDevice(&dev));
  int rc;
  uint64_t* scratch = noalloc_scratch_ptr(dev, &rc);
  if (!scratch) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t W = (size_bits + 63) / 64, NB = W >> 3;
  const uint64_t tiles = (NB + 1 + BVT_SB - 1) / BVT_SB;
  uint32_t* counter = (uint32_t*)scratch;
  uint64_t* status = scratch + 1;
  unsigned long long* info = (unsigned long long*)(scratch + 1 + NOALLOC_TILES);
  uint32_t* err = (uint32_t*)(scratch + 1 + NOALLOC_TILES + INF_N);
  // the array keeps the previous call's contents: clear what must start at 0
  WTG_CK(cudaMemsetAsync(scratch, 0, (1 + tiles) * sizeof(uint64_t), s));
  WTG_CK(cudaMemsetAsync(info, 0, (INF_N + 1) * sizeof(uint64_t), s));
  bv_pass_kernel<<<(unsigned)tiles, BV_THREADS, 0, s>>>(d_words, size_bits, W, NB, WTG_RANK, d_rank, nullptr, 0,
                                                       nullptr, nullptr, nullptr, nullptr, info, status, counter, err);
  count_launch();
  WTG_CK(cudaGetLastError());
  // read the error word on the caller's stream only: no device-wide wait
  uint32_t e = 0;
  WTG_CK(cudaMemcpyAsync(&e, err, sizeof(e), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  if (e) return fail(WTG_ERR_TIMEOUT, "a device-side wait of the rank pass timed out; the table is invalid");
  return WTG_OK;
}

