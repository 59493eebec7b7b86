// wtg_serialize.cu -- sdsl serialize() byte streams of the built structures.
//
// sdsl consumers store and load these structures with serialize()/load()
// (the reference's own parity check compares such files byte for byte,
// wt_int/compareResults.py).  The streams written here are, field for field:
//   wt_int<>::serialize          wt_int/wt_int_par.hpp:887-899
//     m_size (u64), m_sigma (u64), m_tree (bit_vector), m_tree_rank,
//     m_tree_select1, m_tree_select0, m_max_level (u32)
//   rank_support_v<1>::serialize rank/rank_support_v_par.hpp:154-164
//     m_basic_block (int_vector<64>)
//   select_support_mcl::serialize select/select_support_mcl_par.hpp:644-681
//     m_arg_cnt (u64); when non-zero: m_superblock (int_vector<0>), the
//     mini-or-long bit_vector (bit i set when superblock i has a mini block;
//     empty when there are no long blocks), then per superblock its long or
//     mini block (int_vector<0>)
// with every int_vector written as sdsl does: its size in bits (u64), its
// width (one byte, run-time width only), then its ceil(bits/64) words.
//
// The level bits, the rank table and m_superblock go from device memory
// straight into the caller's buffer; the per-superblock blocks are
// interleaved with their 9-byte headers on the host from one copy of the
// block pool.  wt_int's m_sigma (the number of non-empty leaves,
// wt_int_par.hpp:225-240) is counted on the device from the rank table.
#include <cstring>
#include <vector>

#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {

namespace {

// leaves of the tree = both children of every node of the last level that
// holds a zero (left leaf) or a one (right leaf) in its range
__global__ void leaf_count_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                  const uint32_t* __restrict__ C, uint64_t n, int L,
                                  unsigned long long* __restrict__ out) {
  const uint64_t m = 1ull << (L - 1);   // nodes of level L-1
  const uint64_t first = m - 1;         // heap id of its node 0
  const uint64_t off = (uint64_t)(L - 1) * n;
  unsigned long long cnt = 0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m;
       p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t st = C[first + p];
    const uint64_t en = (p + 1 < m) ? C[first + p + 1] : n;
    if (en > st) {
      const uint64_t ones = rank1_dev(rt, tree, off + en) - rank1_dev(rt, tree, off + st);
      cnt += (ones > 0) + (ones < en - st);
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, cnt);
}

// Byte stream being written (or only measured when dst is NULL).
struct Sink {
  uint8_t* dst = nullptr;
  uint64_t off = 0;
  void bytes(const void* p, uint64_t n) {
    if (dst && n) memcpy(dst + off, p, n);
    off += n;
  }
  template <typename T>
  void member(T v) {
    bytes(&v, sizeof(T));
  }
  // int_vector header: size in bits, then the width for run-time widths
  void header(uint64_t bits, int width) {
    member<uint64_t>(bits);
    if (width >= 0) member<uint8_t>((uint8_t)width);
  }
  int device(const void* d, uint64_t n, cudaStream_t s) {
    if (dst && n) WTG_CK(cudaMemcpyAsync(dst + off, d, n, cudaMemcpyDeviceToHost, s));
    off += n;
    return WTG_OK;
  }
};

uint64_t rank_table_words(uint64_t size) {
  if (size == 0) return 2;
  const uint64_t cap = (size + 63) / 64 * 64;
  return ((cap >> 9) + 1) << 1;
}

int put_rank(Sink& o, const BvSupport& bv, cudaStream_t s) {
  const uint64_t words = rank_table_words(bv.size);
  o.header(words * 64, -1);
  return o.device(bv.rank.p, words * 8, s);
}

int put_select(Sink& o, const BvSupport& bv, int t_b, cudaStream_t s) {
  const SelectDev& sd = bv.sel[t_b];
  o.member<uint64_t>(sd.arg_cnt);
  if (!sd.arg_cnt) return WTG_OK;
  const uint64_t nsb = sd.nsb;
  if (sd.sb_nwords != (nsb * sd.logn + 63) / 64) return fail(WTG_ERR_CUDA, "select superblock words inconsistent");
  o.header(nsb * sd.logn, (int)sd.logn);
  int rc;
  if ((rc = o.device(sd.sb_words.p, sd.sb_nwords * 8, s))) return rc;
  const uint64_t flag_words = (nsb + 63) / 64;
  if (!o.dst) {  // lengths only
    o.header(sd.has_long ? nsb : 0, -1);
    o.off += (sd.has_long ? flag_words * 8 : 0) + 9 * nsb + 8 * sd.pool_nwords;
    return WTG_OK;
  }
  std::vector<uint64_t> desc(nsb), pool(sd.pool_nwords);
  WTG_CK(cudaMemcpyAsync(desc.data(), sd.desc.p, nsb * 8, cudaMemcpyDeviceToHost, s));
  if (sd.pool_nwords) WTG_CK(cudaMemcpyAsync(pool.data(), sd.pool.p, sd.pool_nwords * 8, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  if (sd.has_long) {
    std::vector<uint64_t> mini(flag_words, 0);
    for (uint64_t i = 0; i < nsb; ++i)
      if (!((desc[i] >> 7) & 1)) mini[i >> 6] |= 1ull << (i & 63);
    o.header(nsb, -1);
    o.bytes(mini.data(), flag_words * 8);
  } else {
    o.header(0, -1);
  }
  for (uint64_t i = 0; i < nsb; ++i) {
    const uint64_t w = desc[i] & 0x7F, entries = ((desc[i] >> 7) & 1) ? 4096 : 64;
    const uint64_t at = desc[i] >> 8, words = entries * w / 64;
    if (at + words > sd.pool_nwords) return fail(WTG_ERR_CUDA, "select block outside its pool");
    o.header(entries * w, (int)w);
    o.bytes(pool.data() + at, words * 8);
  }
  return WTG_OK;
}

int finish(Sink& o, uint64_t cap, uint64_t* len, cudaStream_t s) {
  if (o.dst) WTG_CK(cudaStreamSynchronize(s));
  (void)cap;
  *len = o.off;
  return WTG_OK;
}

}  // namespace

int tree_leaf_count(TreeImpl& t, uint64_t* sigma, cudaStream_t s) {
  int rc;
  *sigma = 0;
  if (t.n == 0) return WTG_OK;
  if (!(t.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "counting the leaves needs WTG_RANK");
  if ((rc = t.qout.ensure(sizeof(unsigned long long), s))) return rc;
  WTG_CK(cudaMemsetAsync(t.qout.p, 0, sizeof(unsigned long long), s));
  const uint64_t m = 1ull << (t.levels - 1);
  const unsigned grid = (unsigned)std::min<uint64_t>((m + 255) / 256, 1024);
  const uint64_t heap = 1ull << t.levels;
  leaf_count_kernel<<<grid, 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                         t.zeros.as<uint32_t>() + 2 * heap, t.n, t.levels,
                                         t.qout.as<unsigned long long>());
  count_launch();
  WTG_CK(cudaGetLastError());
  WTG_CK(cudaMemcpyAsync(sigma, t.qout.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  return WTG_OK;
}

int tree_serialize(TreeImpl& t, uint8_t* dst, uint64_t cap, uint64_t* len) {
  int rc;
  cudaStream_t s = t.stream;
  Sink o;
  if (t.n == 0) {  // the reference returns from its constructor before anything is built
    o.dst = dst;
    if (dst && cap < 52) return fail(WTG_ERR_INVALID, "cap is smaller than the stream");
    o.member<uint64_t>(0);  // size
    o.member<uint64_t>(0);  // sigma
    o.header(0, -1);        // tree
    o.header(0, -1);        // tree_rank (no table)
    o.member<uint64_t>(0);  // tree_select_1: no args
    o.member<uint64_t>(0);  // tree_select_0
    o.member<uint32_t>(0);  // max_level
    *len = o.off;
    return WTG_OK;
  }
  if ((t.flags & WTG_ALL) != WTG_ALL) return fail(WTG_ERR_INVALID, "wt_int's stream needs WTG_ALL supports");
  // measure first, then write
  Sink m;
  m.member<uint64_t>(0);
  m.member<uint64_t>(0);
  m.header(t.n * (uint64_t)t.levels, -1);
  m.off += t.bit_words * 8;
  if ((rc = put_rank(m, t.bv, s))) return rc;
  if ((rc = put_select(m, t.bv, 1, s))) return rc;
  if ((rc = put_select(m, t.bv, 0, s))) return rc;
  m.member<uint32_t>(0);
  if (!dst) {
    *len = m.off;
    return WTG_OK;
  }
  if (cap < m.off) return fail(WTG_ERR_INVALID, "cap is smaller than the stream");
  uint64_t sigma = 0;
  if ((rc = tree_leaf_count(t, &sigma, s))) return rc;
  o.dst = dst;
  o.member<uint64_t>(t.n);
  o.member<uint64_t>(sigma);
  o.header(t.n * (uint64_t)t.levels, -1);
  if ((rc = o.device(t.bits.p, t.bit_words * 8, s))) return rc;
  if ((rc = put_rank(o, t.bv, s))) return rc;
  if ((rc = put_select(o, t.bv, 1, s))) return rc;
  if ((rc = put_select(o, t.bv, 0, s))) return rc;
  o.member<uint32_t>((uint32_t)t.levels);
  return finish(o, cap, len, s);
}

int bv_serialize(BvSupport& bv, uint32_t part, uint8_t* dst, uint64_t cap, uint64_t* len, cudaStream_t s) {
  int rc;
  if (part != WTG_RANK && part != WTG_SELECT1 && part != WTG_SELECT0)
    return fail(WTG_ERR_INVALID, "part must be one of WTG_RANK, WTG_SELECT1, WTG_SELECT0");
  if (!(bv.flags & part)) return fail(WTG_ERR_INVALID, "that support was not built");
  Sink m;
  if (part == WTG_RANK) rc = put_rank(m, bv, s);
  else rc = put_select(m, bv, part == WTG_SELECT1 ? 1 : 0, s);
  if (rc) return rc;
  if (!dst) {
    *len = m.off;
    return WTG_OK;
  }
  if (cap < m.off) return fail(WTG_ERR_INVALID, "cap is smaller than the stream");
  Sink o;
  o.dst = dst;
  if (part == WTG_RANK) rc = put_rank(o, bv, s);
  else rc = put_select(o, bv, part == WTG_SELECT1 ? 1 : 0, s);
  if (rc) return rc;
  return finish(o, cap, len, s);
}

}  // namespace wtg
