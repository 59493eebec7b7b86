// ref_wt_int_shim.cpp -- runs the reference's own sdsl::wt_int (construction
// and every query method) over a C ABI, so the tests can pin the oracle's
// wt_int queries -- access/rank/select/inverse_select and the range queries
// interval_symbols, lex_count, lex_smaller_count, range_search_2d, expand --
// against it.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file with the
// read-only reference checkout's wt_int/ directory and this directory's
// sdsl_shim/ (a stand-in for the absent sdsl-lite types) on the include path;
// the result goes to oracle/_ref/ and is never shipped.  Positions, ranks and
// symbols cross the ABI as uint64.
#include <algorithm>
#include <atomic>
#include <cassert>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <sdsl/int_vector.hpp>
#include <sdsl/rank_support.hpp>
#include <sdsl/select_support.hpp>
#include <sdsl/util.hpp>
#include <sdsl/sdsl_concepts.hpp>
#include <sdsl/wt_helper.hpp>

// the reference class keeps its bitvector and supports in protected members
#define private public
#define protected public
#include "wt_int_par.hpp"
#undef private
#undef protected

namespace {

typedef sdsl::wt_int<sdsl::bit_vector, sdsl::rank_support_v<1, 1>, sdsl::select_support_mcl<1, 1>,
                     sdsl::select_support_mcl<0, 1>>
    wt_t;

template <uint8_t W, class T>
wt_t* build(const T* seq, uint64_t n, uint32_t max_level) {
  sdsl::int_vector<W> buf(n, 0, W);
  for (uint64_t i = 0; i < n; ++i) buf[i] = (uint64_t)seq[i];
  return new wt_t(buf, n, max_level);
}

}  // namespace

extern "C" {

// wt_int(buf, n, max_level) (wt_int_par.hpp:368-406) over n symbols of
// elem_bytes (1, 2, 4 or 8) bytes; NULL when the constructor throws.
void* ref_wtint_new(const void* seq, int elem_bytes, uint64_t n, uint32_t max_level) {
  try {
    switch (elem_bytes) {
      case 1: return build<8>((const uint8_t*)seq, n, max_level);
      case 2: return build<16>((const uint16_t*)seq, n, max_level);
      case 4: return build<32>((const uint32_t*)seq, n, max_level);
      case 8: return build<64>((const uint64_t*)seq, n, max_level);
    }
  } catch (...) {
  }
  return nullptr;
}

void ref_wtint_free(void* h) { delete (wt_t*)h; }

// wt_int::serialize (wt_int_par.hpp:887-899) into dst when it holds cap >=
// the stream's length bytes; returns that length (dst may be NULL)
uint64_t ref_wtint_serialize(void* h, uint8_t* dst, uint64_t cap) {
  std::ostringstream os;
  ((const wt_t*)h)->serialize(os);
  const std::string b = os.str();
  if (dst && cap >= b.size()) memcpy(dst, b.data(), b.size());
  return b.size();
}

// wt_int::load (wt_int_par.hpp:902-911) from len bytes; NULL when the
// stream ends early
void* ref_wtint_load(const uint8_t* src, uint64_t len) {
  std::istringstream is(std::string((const char*)src, len));
  wt_t* w = new wt_t();
  w->load(is);
  if (is.fail()) {
    delete w;
    return nullptr;
  }
  return w;
}

// size, sigma, max_level, words of m_tree
void ref_wtint_info(void* h, uint64_t* out) {
  const wt_t* w = (const wt_t*)h;
  out[0] = w->m_size;
  out[1] = w->m_sigma;
  out[2] = w->m_max_level;
  out[3] = (w->m_tree.bit_size() + 63) >> 6;
}

void ref_wtint_bits(void* h, uint64_t* out) {
  const wt_t* w = (const wt_t*)h;
  memcpy(out, w->m_tree.data(), ((w->m_tree.bit_size() + 63) >> 6) * 8);
}

uint64_t ref_wtint_access(void* h, uint64_t i) { return (*(const wt_t*)h)[i]; }
uint64_t ref_wtint_rank(void* h, uint64_t i, uint64_t c) { return ((const wt_t*)h)->rank(i, c); }

void ref_wtint_inverse_select(void* h, uint64_t i, uint64_t* out) {
  auto r = ((const wt_t*)h)->inverse_select(i);
  out[0] = r.first;
  out[1] = r.second;
}

// select(i, c); ~0 when the reference throws (c does not occur i times)
uint64_t ref_wtint_select(void* h, uint64_t i, uint64_t c) {
  try {
    return ((const wt_t*)h)->select(i, c);
  } catch (const std::logic_error&) {
    return ~0ull;
  }
}

// out = (rank(i, c), smaller, greater) (wt_int_par.hpp:715-745)
void ref_wtint_lex_count(void* h, uint64_t i, uint64_t j, uint64_t c, uint64_t* out) {
  auto t = ((const wt_t*)h)->lex_count(i, j, c);
  out[0] = std::get<0>(t);
  out[1] = std::get<1>(t);
  out[2] = std::get<2>(t);
}

// out = (rank(i, c), smaller) (wt_int_par.hpp:758-782)
void ref_wtint_lex_smaller_count(void* h, uint64_t i, uint64_t c, uint64_t* out) {
  auto t = ((const wt_t*)h)->lex_smaller_count(i, c);
  out[0] = std::get<0>(t);
  out[1] = std::get<1>(t);
}

// interval_symbols(i, j) (wt_int_par.hpp:684-702): returns k; cs, rank_i,
// rank_j hold cap >= min(2^max_level, j - i) entries
uint64_t ref_wtint_interval_symbols(void* h, uint64_t i, uint64_t j, uint64_t cap, uint64_t* cs, uint64_t* ri,
                                    uint64_t* rj) {
  std::vector<uint64_t> vc(cap), vi(cap), vj(cap);
  uint64_t k = 0;
  ((const wt_t*)h)->interval_symbols(i, j, k, vc, vi, vj);
  std::copy(vc.begin(), vc.begin() + k, cs);
  std::copy(vi.begin(), vi.begin() + k, ri);
  std::copy(vj.begin(), vj.begin() + k, rj);
  return k;
}

// range_search_2d(lb, rb, vlb, vrb, report) (wt_int_par.hpp:801-815): returns
// the count; with report, the first min(count, cap) points (position, value)
// in the reference's order
uint64_t ref_wtint_range_search_2d(void* h, uint64_t lb, uint64_t rb, uint64_t vlb, uint64_t vrb, int report,
                                   uint64_t cap, uint64_t* pos, uint64_t* val) {
  auto r = ((const wt_t*)h)->range_search_2d(lb, rb, vlb, vrb, report != 0);
  const uint64_t m = std::min<uint64_t>(cap, r.second.size());
  for (uint64_t q = 0; q < m; ++q) {
    pos[q] = r.second[q].first;
    val[q] = r.second[q].second;
  }
  return r.first;
}

// expand(v) (wt_int_par.hpp:966-984): v and the two children as
// (offset, size, level, sym)
void ref_wtint_expand(void* h, const uint64_t* v, uint64_t* left, uint64_t* right) {
  wt_t::node_type nv(v[0], v[1], v[2], v[3]);
  auto r = ((const wt_t*)h)->expand(nv);
  left[0] = r.first.offset;
  left[1] = r.first.size;
  left[2] = r.first.level;
  left[3] = r.first.sym;
  right[0] = r.second.offset;
  right[1] = r.second.size;
  right[2] = r.second.level;
  right[3] = r.second.sym;
}

// expand(v, ranges) (wt_int_par.hpp:1027-1048): nr closed ranges
// [s, e] (2 words each) -> left and right child ranges
void ref_wtint_expand_ranges(void* h, const uint64_t* v, const uint64_t* ranges, uint64_t nr, uint64_t* left,
                             uint64_t* right) {
  wt_t::node_type nv(v[0], v[1], v[2], v[3]);
  sdsl::range_vec_type rv(nr);
  for (uint64_t q = 0; q < nr; ++q) rv[q] = sdsl::range_type(ranges[2 * q], ranges[2 * q + 1]);
  auto r = ((const wt_t*)h)->expand(nv, rv);
  for (uint64_t q = 0; q < nr; ++q) {
    left[2 * q] = r.first[q].first;
    left[2 * q + 1] = r.first[q].second;
    right[2 * q] = r.second[q].first;
    right[2 * q + 1] = r.second[q].second;
  }
}
}
