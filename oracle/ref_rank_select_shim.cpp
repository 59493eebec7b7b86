// ref_rank_select_shim.cpp -- runs the reference's own rank_support_v_par and
// select_support_mcl_par construction/query code over a C ABI, so the tests
// can pin the oracle's rank tables and select samples against it.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file with the
// read-only reference checkout's select/ directory and this directory's
// sdsl_shim/ (a stand-in for the absent sdsl-lite types) on the include path;
// the result goes to oracle/_ref/ and is never shipped.
//
// The select structure is exported in the flat packed layout the oracle and
// the GPU library use: m_superblock's int_vector<0> words, one descriptor per
// superblock ((pool word offset << 8) | (is_long << 7) | width) and a pool
// holding every long or mini block's int_vector<0> words in superblock order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cassert>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <sdsl/int_vector.hpp>
#include <sdsl/rank_support.hpp>
#include <sdsl/select_support.hpp>
#include <sdsl/util.hpp>

// the reference classes keep their tables in private members
#define private public
#define protected public
#include "select_support_mcl_par.hpp"
#undef private
#undef protected

namespace {

sdsl::bit_vector make_bv(const uint64_t* words, uint64_t size) {
  sdsl::bit_vector bv(size, 0);
  uint64_t nw = (size + 63) / 64;
  if (nw) memcpy(bv.data(), words, nw * 8);
  if (size & 63) bv.data()[nw - 1] &= sdsl::bits::lo_set_f((uint32_t)(size & 63));
  return bv;
}

struct sel_any {
  virtual ~sel_any() {}
  virtual void info(uint64_t* out) = 0;
  virtual void copy(uint64_t* sb_words, uint64_t* desc, uint64_t* pool) = 0;
  virtual uint64_t query(uint64_t i) = 0;
  virtual std::string serialize() = 0;
};

template <uint8_t t_b>
struct sel_impl : sel_any {
  sdsl::bit_vector bv;
  sdsl::select_support_mcl<t_b, 1>* ss;
  sel_impl(const uint64_t* words, uint64_t size) : bv(make_bv(words, size)) {
    ss = new sdsl::select_support_mcl<t_b, 1>(&bv);
  }
  // over a bit_vector the caller keeps alive (no copy)
  sel_impl(const uint64_t*, uint64_t, const sdsl::bit_vector* ext) {
    ss = new sdsl::select_support_mcl<t_b, 1>(ext);
  }
  ~sel_impl() { delete ss; }
  uint64_t nsb() const { return (ss->m_arg_cnt + 4095) >> 12; }
  bool is_long(uint64_t i) const {
    return ss->m_longsuperblock != nullptr && !ss->m_longsuperblock[i].empty();
  }
  const sdsl::int_vector<0>& block(uint64_t i) const {
    return is_long(i) ? ss->m_longsuperblock[i] : ss->m_miniblock[i];
  }
  static uint64_t words_of(const sdsl::int_vector<0>& v) { return (v.bit_size() + 63) >> 6; }
  void info(uint64_t* out) override {
    uint64_t pool = 0;
    for (uint64_t i = 0; i < nsb(); ++i) pool += words_of(block(i));
    out[0] = bv.size();
    out[1] = ss->m_arg_cnt;
    out[2] = ss->m_logn;
    out[3] = ss->m_logn4;
    out[4] = nsb();
    out[5] = ss->m_longsuperblock != nullptr;
    out[6] = ss->m_arg_cnt ? words_of(ss->m_superblock) : 0;
    out[7] = pool;
  }
  void copy(uint64_t* sb_words, uint64_t* desc, uint64_t* pool) override {
    if (ss->m_arg_cnt == 0) return;
    memcpy(sb_words, ss->m_superblock.data(), words_of(ss->m_superblock) * 8);
    uint64_t off = 0;
    for (uint64_t i = 0; i < nsb(); ++i) {
      const sdsl::int_vector<0>& b = block(i);
      desc[i] = (off << 8) | ((uint64_t)is_long(i) << 7) | b.width();
      memcpy(pool + off, b.data(), words_of(b) * 8);
      off += words_of(b);
    }
  }
  uint64_t query(uint64_t i) override { return ss->select(i); }
  std::string serialize() override {
    std::ostringstream os;
    ss->serialize(os);
    return os.str();
  }
};

uint64_t emit(const std::string& b, uint8_t* dst, uint64_t cap) {
  if (dst && cap >= b.size()) memcpy(dst, b.data(), b.size());
  return b.size();
}

}  // namespace

extern "C" {

// rank_support_v<1> over the first `size` bits of `words`; copies m_basic_block.
int ref_rank_build(const uint64_t* words, uint64_t size, uint64_t* tbl, uint64_t tbl_words) {
  sdsl::bit_vector bv = make_bv(words, size);
  sdsl::rank_support_v<1, 1> rs(&bv);
  if (rs.m_basic_block.size() != tbl_words) return -1;
  memcpy(tbl, rs.m_basic_block.data(), tbl_words * 8);
  return 0;
}

uint64_t ref_rank_query(const uint64_t* words, uint64_t size, uint64_t idx) {
  sdsl::bit_vector bv = make_bv(words, size);
  sdsl::rank_support_v<1, 1> rs(&bv);
  return rs.rank(idx);
}

void* ref_select_new(const uint64_t* words, uint64_t size, int t_b) {
  if (t_b) return new sel_impl<1>(words, size);
  return new sel_impl<0>(words, size);
}
void ref_select_info(void* h, uint64_t* info) { ((sel_any*)h)->info(info); }
void ref_select_copy(void* h, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  ((sel_any*)h)->copy(sb_words, desc, pool);
}
uint64_t ref_select_query(void* h, uint64_t i) { return ((sel_any*)h)->query(i); }
void ref_select_free(void* h) { delete (sel_any*)h; }

// rank_support_v::serialize (rank/rank_support_v_par.hpp:154-164) of the
// table over the first `size` bits of `words`; returns the stream length and
// fills dst when cap suffices (dst may be NULL)
uint64_t ref_rank_serialize(const uint64_t* words, uint64_t size, uint8_t* dst, uint64_t cap) {
  sdsl::bit_vector bv = make_bv(words, size);
  sdsl::rank_support_v<1, 1> rs(&bv);
  std::ostringstream os;
  rs.serialize(os);
  return emit(os.str(), dst, cap);
}

// Seconds of the rank_support_v<1>, select_support_mcl<1> and
// select_support_mcl<0> constructors over the first `size` bits of `words`
// (the timed CPU baseline; the bit_vector is filled before the clock
// starts): out = {t_rank, t_select1, t_select0, select1 words, select0
// words}, the words being m_superblock's plus every block's.
void ref_rank_select_time(const uint64_t* words, uint64_t size, double* out) {
  sdsl::bit_vector bv = make_bv(words, size);
  auto t0 = std::chrono::steady_clock::now();
  { sdsl::rank_support_v<1, 1> rs(&bv); }
  auto t1 = std::chrono::steady_clock::now();
  out[0] = std::chrono::duration<double>(t1 - t0).count();
  for (int t_b = 1; t_b >= 0; --t_b) {
    sel_any* h = nullptr;
    t0 = std::chrono::steady_clock::now();
    if (t_b) h = new sel_impl<1>(words, size, &bv);
    else h = new sel_impl<0>(words, size, &bv);
    t1 = std::chrono::steady_clock::now();
    uint64_t info[8];
    h->info(info);
    out[t_b ? 1 : 2] = std::chrono::duration<double>(t1 - t0).count();
    out[t_b ? 3 : 4] = (double)(info[6] + info[4] + info[7]);
    delete h;
  }
}

// Seconds of the rank_support_v<1>, select_support_mcl<1> and <0>
// constructors over T bitvectors (bitvector t: sizes[t] bits at word
// woffs[t] of words), the bitvectors spread over the OpenMP threads; the
// bit_vectors are filled before the clock starts.
double ref_rank_select_batch_time(const uint64_t* words, const uint64_t* woffs, const uint64_t* sizes, uint64_t T) {
  std::vector<sdsl::bit_vector> bvs;
  bvs.reserve(T);
  for (uint64_t t = 0; t < T; ++t) bvs.push_back(make_bv(words + woffs[t], sizes[t]));
  const auto t0 = std::chrono::steady_clock::now();
#if defined(OPENMP)
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (long t = 0; t < (long)T; ++t) {
    sdsl::rank_support_v<1, 1> rs(&bvs[t]);
    sdsl::select_support_mcl<1, 1> s1(&bvs[t]);
    sdsl::select_support_mcl<0, 1> s0(&bvs[t]);
  }
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// select(q[i]) for nq queries on a select structure (OpenMP over the
// queries); returns the seconds
double ref_select_batch(void* h, const uint64_t* q, uint64_t nq, uint64_t* out) {
  sel_any* s = (sel_any*)h;
  const auto t0 = std::chrono::steady_clock::now();
#if defined(OPENMP)
#pragma omp parallel for schedule(static, 4096)
#endif
  for (long i = 0; i < (long)nq; ++i) out[i] = s->query(q[i]);
  const auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// select_support_mcl::serialize (select/select_support_mcl_par.hpp:644-681)
uint64_t ref_select_serialize(void* h, uint8_t* dst, uint64_t cap) {
  return emit(((sel_any*)h)->serialize(), dst, cap);
}
}
