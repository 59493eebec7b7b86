// wtg_reference_api.hpp -- the reference's C++ interface for the
// wavelet-tree path, backed by libwtg (include/wtg.h).
//
// Header-only.  Include it instead of compiling wavelet/levelWT/WT.C (or
// ddWT/recWT/serialWT) and instead of the rank/select/wt_int "_par" headers;
// link with -lwtg.  Names, argument meaning and ownership follow the
// reference:
//   * WT(symbol* s, uintT n, uintT sigma) -> pair<WTnode*, long*>
//     (wavelet/levelWT/WT.h:30-43): outputs are malloc'ed, freed by the caller
//     with free() (levelWT/WTTime.C:99,135); `symbol`, `uintT` and the WTnode
//     field width follow the same -DINT / -DLONG knobs (parallel.h:71-81).
//   * wtg::wt_int (sdsl::wt_int<>, wt_int/wt_int_par.hpp:368-1048): operator[],
//     rank, inverse_select, select, size, and the range queries
//     interval_symbols, lex_count, lex_smaller_count, range_search_2d, root,
//     expand; std::logic_error where the reference throws one
//     (wt_int_par.hpp:377,645).
//   * wtg::rank_support_v / wtg::select_support_mcl<t_b>
//     (rank/rank_support_v_par.hpp:69-142, select/select_support_mcl_par.hpp:
//     120-129,564-611) over a bit vector given as 64-bit words.
//   * serialize(std::ostream&) on all three, writing sdsl's byte streams
//     (wt_int_par.hpp:887-899, rank_support_v_par.hpp:154-164,
//     select_support_mcl_par.hpp:644-681), and wtg::store_to_file.
// Every call runs on the current CUDA device; failures other than the
// reference's own exceptions raise std::runtime_error with wtg_last_error().
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <ostream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/wtg.h"

#ifndef WTG_NO_REFERENCE_TYPES
#if defined(LONG)
typedef unsigned long uintT;
#else
typedef unsigned int uintT;
#endif
#ifdef INT
typedef uintT symbol;
#else
typedef unsigned char symbol;
#endif
typedef uintT intOffset;
struct WTnode {
  intOffset bitmapPtr;
  uintT length;
  uintT parent, leftChild, rightChild;
};
#endif

namespace wtg {

inline void check(int rc) {
  if (rc != WTG_OK) throw std::runtime_error(std::string("wtg: ") + wtg_last_error());
}

// max(1, log2Up(sigma)) (wavelet/levelWT/WT.C:53)
inline int levels_for_sigma(uint64_t sigma) {
  int a = 0;
  for (uint64_t b = sigma - 1; b > 0; b >>= 1) ++a;
  return a < 1 ? 1 : a;
}

// Writes the stream `fill(dst, cap, len)` produces (dst NULL: length only) to
// `out`; returns the bytes written, as sdsl's serialize() does.
template <typename F>
inline uint64_t write_stream(std::ostream& out, F fill) {
  uint64_t len = 0;
  check(fill(nullptr, 0, &len));
  std::vector<char> buf(len);
  check(fill(buf.data(), len, &len));
  out.write(buf.data(), (std::streamsize)len);
  return len;
}

// Owning handle of a GPU-built tree.
class tree {
 public:
  tree() = default;
  tree(const void* seq, uint64_t n, int elem_bytes, int levels, uint32_t flags) {
    check(wtg_tree_build(seq, n, elem_bytes, levels, flags, &t_));
    check(wtg_tree_info(t_, info_));
  }
  tree(const tree&) = delete;
  tree& operator=(const tree&) = delete;
  tree(tree&& o) noexcept : t_(o.t_) {
    std::memcpy(info_, o.info_, sizeof(info_));
    o.t_ = nullptr;
  }
  tree& operator=(tree&& o) noexcept {
    if (this != &o) {
      wtg_tree_free(t_);
      t_ = o.t_;
      std::memcpy(info_, o.info_, sizeof(info_));
      o.t_ = nullptr;
    }
    return *this;
  }
  ~tree() { wtg_tree_free(t_); }
  wtg_tree* get() const { return t_; }
  uint64_t n() const { return info_[0]; }
  int levels() const { return (int)info_[1]; }
  uint64_t bit_words() const { return info_[2]; }
  uint64_t rank_words() const { return info_[3]; }

 private:
  wtg_tree* t_ = nullptr;
  uint64_t info_[4] = {0, 0, 0, 0};
};

// sdsl::wt_int<> (wt_int/wt_int_par.hpp): level bits, rank_support_v and
// select_support_mcl<1>/<0> over them, built on the GPU.
class wt_int {
 public:
  typedef uint64_t size_type;
  typedef uint64_t value_type;
  typedef std::pair<value_type, size_type> point_type;  // (position, value)
  typedef std::vector<point_type> point_vec_type;
  typedef std::pair<size_type, point_vec_type> r2d_res_type;
  typedef std::pair<size_type, size_type> range_type;  // closed [first, second]
  typedef std::vector<range_type> range_vec_type;
  // a node of the tree (wt_int_par.hpp:914-960): its bit offset, size, level
  // and the symbol prefix of its path
  struct node_type {
    size_type offset = 0, size = 0, level = 0;
    value_type sym = 0;
    node_type(size_type o = 0, size_type sz = 0, size_type l = 0, value_type sy = 0)
        : offset(o), size(sz), level(l), sym(sy) {}
    bool operator==(const node_type& v) const { return offset == v.offset; }
    bool operator<(const node_type& v) const { return offset < v.offset; }
    bool operator>(const node_type& v) const { return offset > v.offset; }
  };
  wt_int() = default;
  // wt_int(buf, size, max_level) (wt_int_par.hpp:368-406); max_level 0 derives
  // hi(max(1, max symbol)) + 1
  template <typename T>
  wt_int(const std::vector<T>& buf, size_type size, uint32_t max_level = 0) {
    if (buf.size() < size)
      throw std::logic_error("n=" + std::to_string(buf.size()) + " < " + std::to_string(size) + "=m_size");
    if (size) t_ = tree(buf.data(), size, (int)sizeof(T), (int)max_level, WTG_ALL);
  }
  size_type size() const { return t_.n(); }
  bool empty() const { return size() == 0; }
  uint32_t max_level() const { return (uint32_t)t_.levels(); }

  value_type operator[](size_type i) const {
    uint64_t out = 0;
    check(wtg_query_access(t_.get(), &i, 1, &out));
    return out;
  }
  size_type rank(size_type i, value_type c) const {
    uint64_t out = 0;
    check(wtg_query_rank(t_.get(), &i, &c, 1, &out));
    return out;
  }
  std::pair<size_type, value_type> inverse_select(size_type i) const {
    uint64_t r = 0, c = 0;
    check(wtg_query_inverse_select(t_.get(), &i, 1, &r, &c));
    return std::make_pair(r, c);
  }
  size_type select(size_type i, value_type c) const {
    uint64_t out = 0;
    check(wtg_query_select(t_.get(), &i, &c, 1, &out));
    if (out == ~0ull)
      throw std::logic_error("select(" + std::to_string(i) + "," + std::to_string(c) +
                             "): c does not occur i times in the WT");
    return out;
  }
  // batched forms (one kernel launch for many queries)
  void access(const uint64_t* idx, uint64_t nq, uint64_t* out) const {
    check(wtg_query_access(t_.get(), idx, nq, out));
  }
  void rank(const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out) const {
    check(wtg_query_rank(t_.get(), idx, sym, nq, out));
  }
  // interval_symbols (wt_int_par.hpp:684-702): the k distinct symbols of
  // [i, j) in cs[0..k-1], increasing, with rank(i, c) and rank(j, c); the
  // vectors hold at least k entries (sigma is enough)
  void interval_symbols(size_type i, size_type j, size_type& k, std::vector<value_type>& cs,
                        std::vector<size_type>& rank_c_i, std::vector<size_type>& rank_c_j) const {
    if (i > j || j > size()) throw std::logic_error("interval_symbols: need i <= j <= size()");
    uint64_t kk = 0;
    check(wtg_query_interval_symbols(t_.get(), &i, &j, 1, &kk, 0, nullptr, nullptr, nullptr));
    k = kk;
    if (!kk) return;
    if (cs.size() < kk || rank_c_i.size() < kk || rank_c_j.size() < kk)
      throw std::logic_error("interval_symbols: output vectors shorter than the symbol count");
    check(wtg_query_interval_symbols(t_.get(), &i, &j, 1, &kk, kk, cs.data(), rank_c_i.data(), rank_c_j.data()));
  }
  // lex_count (wt_int_par.hpp:715-745): (rank(i, c), #symbols < c in [i, j),
  // #symbols > c in [i, j))
  std::tuple<size_type, size_type, size_type> lex_count(size_type i, size_type j, value_type c) const {
    uint64_t r = 0, sm = 0, gr = 0;
    check(wtg_query_lex_count(t_.get(), &i, &j, &c, 1, &r, &sm, &gr));
    return std::make_tuple(r, sm, gr);
  }
  // lex_smaller_count (wt_int_par.hpp:758-782): (rank(i, c), #symbols < c in [0, i))
  std::tuple<size_type, size_type> lex_smaller_count(size_type i, value_type c) const {
    uint64_t r = 0, sm = 0;
    check(wtg_query_lex_smaller_count(t_.get(), &i, &c, 1, &r, &sm));
    return std::make_tuple(r, sm);
  }
  // range_search_2d (wt_int_par.hpp:801-815): points of positions [lb, rb]
  // with values in [vlb, vrb], as (position, value), values increasing
  r2d_res_type range_search_2d(size_type lb, size_type rb, value_type vlb, value_type vrb,
                               bool report = true) const {
    uint64_t cnt = 0;
    check(wtg_query_range_search_2d(t_.get(), &lb, &rb, &vlb, &vrb, 1, &cnt, 0, nullptr, nullptr));
    if (cnt == ~0ull) throw std::logic_error("range_search_2d: rb >= size()");
    point_vec_type pts;
    if (report && cnt) {
      std::vector<uint64_t> pos(cnt), val(cnt);
      check(wtg_query_range_search_2d(t_.get(), &lb, &rb, &vlb, &vrb, 1, &cnt, cnt, pos.data(), val.data()));
      pts.reserve(cnt);
      for (uint64_t q = 0; q < cnt; ++q) pts.emplace_back(pos[q], val[q]);
    }
    return r2d_res_type(cnt, std::move(pts));
  }
  node_type root() const { return node_type(0, size(), 0, 0); }
  bool is_leaf(const node_type& v) const { return v.level == max_level(); }
  value_type sym(const node_type& v) const { return v.sym; }
  bool empty(const node_type& v) const { return v.size == 0; }
  // expand(v) (wt_int_par.hpp:966-984): the children of inner node v
  std::pair<node_type, node_type> expand(const node_type& v) const {
    const uint64_t in[4] = {v.offset, v.size, v.level, v.sym};
    uint64_t l[4], r[4];
    check(wtg_query_expand(t_.get(), in, 1, l, r));
    return std::make_pair(node_type(l[0], l[1], l[2], l[3]), node_type(r[0], r[1], r[2], r[3]));
  }
  // expand(v, ranges) (wt_int_par.hpp:1027-1048): each range of v mapped to
  // the left and the right child
  std::pair<range_vec_type, range_vec_type> expand(const node_type& v, const range_vec_type& ranges) const {
    const uint64_t in[4] = {v.offset, v.size, v.level, v.sym};
    std::vector<uint64_t> r(2 * ranges.size()), lo(r.size()), hi(r.size());
    for (size_t q = 0; q < ranges.size(); ++q) {
      r[2 * q] = ranges[q].first;
      r[2 * q + 1] = ranges[q].second;
    }
    check(wtg_query_expand_ranges(t_.get(), in, r.data(), ranges.size(), lo.data(), hi.data()));
    range_vec_type a(ranges.size()), b(ranges.size());
    for (size_t q = 0; q < ranges.size(); ++q) {
      a[q] = range_type(lo[2 * q], lo[2 * q + 1]);
      b[q] = range_type(hi[2 * q], hi[2 * q + 1]);
    }
    return std::make_pair(std::move(a), std::move(b));
  }
  std::pair<range_type, range_type> expand(const node_type& v, const range_type& r) const {
    auto e = expand(v, range_vec_type(1, r));
    return std::make_pair(e.first[0], e.second[0]);
  }
  // wt_int::serialize (wt_int_par.hpp:887-899): sdsl's byte stream
  uint64_t serialize(std::ostream& out) const {
    tree empty;
    wtg_tree* h = t_.get();
    if (!h) {  // the reference serializes an empty wt_int too
      empty = tree(nullptr, 0, 1, 1, WTG_ALL);
      h = empty.get();
    }
    return write_stream(out, [h](void* d, uint64_t c, uint64_t* l) { return wtg_tree_serialize(h, d, c, l); });
  }
  // the concatenated level bitvector (wt_int::tree, wt_int_par.hpp:80,290)
  std::vector<uint64_t> tree_words() const {
    std::vector<uint64_t> w(t_.bit_words());
    check(wtg_tree_get_bits(t_.get(), w.data(), w.size()));
    return w;
  }

 private:
  tree t_;
};

// rank_support_v<1> over a bit vector (rank/rank_support_v_par.hpp:69-142).
class rank_support_v {
 public:
  rank_support_v(const uint64_t* words, uint64_t size_bits) {
    check(wtg_bv_build(words, size_bits, WTG_RANK, &b_));
  }
  rank_support_v(const rank_support_v&) = delete;
  rank_support_v& operator=(const rank_support_v&) = delete;
  ~rank_support_v() { wtg_bv_free(b_); }
  uint64_t rank(uint64_t idx) const {
    uint64_t out = 0;
    check(wtg_bv_rank(b_, &idx, 1, &out));
    return out;
  }
  uint64_t operator()(uint64_t idx) const { return rank(idx); }
  // rank_support_v::serialize (rank_support_v_par.hpp:154-164)
  uint64_t serialize(std::ostream& out) const {
    wtg_bv* b = b_;
    return write_stream(out, [b](void* d, uint64_t c, uint64_t* l) { return wtg_bv_serialize(b, WTG_RANK, d, c, l); });
  }
  // m_basic_block in the reference layout
  std::vector<uint64_t> basic_block() const {
    uint64_t nw = 0;
    check(wtg_bv_rank_words(b_, &nw));
    std::vector<uint64_t> t(nw);
    check(wtg_bv_get_rank(b_, t.data(), nw));
    return t;
  }

 private:
  wtg_bv* b_ = nullptr;
};

// select_support_mcl<t_b> over a bit vector (select/select_support_mcl_par.hpp).
template <uint8_t t_b = 1>
class select_support_mcl {
 public:
  select_support_mcl(const uint64_t* words, uint64_t size_bits) {
    check(wtg_bv_build(words, size_bits, t_b ? WTG_SELECT1 : WTG_SELECT0, &b_));
  }
  select_support_mcl(const select_support_mcl&) = delete;
  select_support_mcl& operator=(const select_support_mcl&) = delete;
  ~select_support_mcl() { wtg_bv_free(b_); }
  // select(i), 1 <= i <= number of args (select_support_mcl_par.hpp:564-611)
  uint64_t select(uint64_t i) const {
    uint64_t out = 0;
    check(wtg_bv_select(b_, t_b, &i, 1, &out));
    return out;
  }
  uint64_t operator()(uint64_t i) const { return select(i); }
  uint64_t arg_cnt() const {
    uint64_t info[8];
    check(wtg_bv_select_info(b_, t_b, info));
    return info[1];
  }
  // select_support_mcl::serialize (select_support_mcl_par.hpp:644-681)
  uint64_t serialize(std::ostream& out) const {
    wtg_bv* b = b_;
    const uint32_t part = t_b ? WTG_SELECT1 : WTG_SELECT0;
    return write_stream(out, [b, part](void* d, uint64_t c, uint64_t* l) { return wtg_bv_serialize(b, part, d, c, l); });
  }

 private:
  wtg_bv* b_ = nullptr;
};

// sdsl's store_to_file(v, file): v's serialize() stream in a file
template <typename T>
inline bool store_to_file(const T& v, const std::string& file) {
  std::ofstream out(file, std::ios::binary | std::ios::trunc);
  if (!out) return false;
  v.serialize(out);
  return (bool)out;
}

}  // namespace wtg

#ifndef WTG_NO_REFERENCE_TYPES
// levelWT's WT() (wavelet/levelWT/WT.h:43, WT.C:43-227): the level-concatenated
// bitvector of ceil(n*levels/64) words and 2*sigma WTnode records, both
// malloc'ed; the caller frees them with free().
inline std::pair<WTnode*, long*> WT(symbol* s, uintT n, uintT sigma) {
  const int levels = wtg::levels_for_sigma(sigma);
  wtg::tree t(s, n, (int)sizeof(symbol), levels, 0);
  const uint64_t nw = t.bit_words();
  long* wt = (long*)std::malloc(sizeof(long) * (nw ? nw : 1));
  WTnode* nodes = (WTnode*)std::malloc(sizeof(WTnode) * 2 * (size_t)sigma);
  if (!wt || !nodes) {
    std::free(wt);
    std::free(nodes);
    throw std::bad_alloc();
  }
  wtg::check(wtg_tree_get_bits(t.get(), (uint64_t*)wt, nw));
  wtg::check(wtg_tree_get_nodes(t.get(), (int)sizeof(uintT), 2 * (uint64_t)sigma, nodes));
  return std::make_pair(nodes, wt);
}
#endif
