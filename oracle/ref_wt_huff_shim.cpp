// ref_wt_huff_shim.cpp -- runs the reference's own Huffman-shaped wavelet tree
// (wt_huff/wt_huff_par.hpp: sdsl::wt_huff, i.e. wt_pc with the Huffman shape,
// built in parallel by wt_huff/wt_pc_par.hpp) over a C ABI, so the tests can
// pin the oracle's Huffman-shaped build against it.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file with the
// read-only reference checkout's wt_huff/ and select/ directories and this
// directory's sdsl_shim/ (a stand-in for the absent sdsl-lite types,
// including the breadth-first byte code tree wt_pc uses) on the include path;
// the result goes to oracle/_ref/ and is never shipped.  As the reference's
// wt_huff/WT.h does, the rank and select "_par" headers come first.
#include <algorithm>
#include <atomic>
#include <cassert>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <queue>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include <sdsl/int_vector.hpp>
#include <sdsl/rank_support.hpp>
#include <sdsl/select_support.hpp>
#include <sdsl/util.hpp>
#include <sdsl/sdsl_concepts.hpp>
#include <sdsl/wt_helper.hpp>

// the reference classes keep their members private
#define private public
#define protected public
#include "select_support_mcl_par.hpp"
#include "wt_huff_par.hpp"
#undef private
#undef protected

namespace {

typedef sdsl::wt_pc<sdsl::huff_shape, sdsl::bit_vector, sdsl::rank_support_v<1, 1>, sdsl::select_support_mcl<1, 1>,
                    sdsl::select_support_mcl<0, 1>, sdsl::byte_tree<>>
    huff_t;

}  // namespace

extern "C" {

// wt_huff(text, n) (wt_huff/wt_pc_par.hpp:321-361) over n bytes; NULL when
// the constructor throws
void* ref_huff_new(const uint8_t* s, uint64_t n) {
  try {
    sdsl::int_vector<8> buf(n, 0, 8);
    for (uint64_t i = 0; i < n; ++i) buf[i] = s[i];
    return new huff_t(buf, n);
  } catch (...) {
  }
  return nullptr;
}

void ref_huff_free(void* h) { delete (huff_t*)h; }

// size, sigma, bit size of m_bv, tree nodes
void ref_huff_info(void* h, uint64_t* out) {
  const huff_t* w = (const huff_t*)h;
  out[0] = w->m_size;
  out[1] = w->m_sigma;
  out[2] = w->m_bv.bit_size();
  out[3] = w->m_tree.size();
}

// m_bv words (ceil(bits / 64)), the rank table (words as returned by
// ref_huff_rank_words), and per node (bv_pos, bv_pos_rank, parent, child0,
// child1), and per byte (c_to_leaf, path)
void ref_huff_bits(void* h, uint64_t* out) {
  const huff_t* w = (const huff_t*)h;
  const uint64_t nw = (w->m_bv.bit_size() + 63) >> 6;
  if (nw) memcpy(out, w->m_bv.data(), nw * 8);
}

uint64_t ref_huff_rank_words(void* h) { return ((const huff_t*)h)->m_bv_rank.m_basic_block.size(); }

void ref_huff_rank(void* h, uint64_t* out) {
  const huff_t* w = (const huff_t*)h;
  const uint64_t m = w->m_bv_rank.m_basic_block.size();
  if (m) memcpy(out, w->m_bv_rank.m_basic_block.data(), m * 8);
}

void ref_huff_nodes(void* h, uint64_t* nodes, uint64_t* leaves, uint64_t* paths) {
  const huff_t* w = (const huff_t*)h;
  for (uint64_t v = 0; v < w->m_tree.size(); ++v) {
    const auto& d = w->m_tree.m_nodes[v];
    nodes[5 * v + 0] = d.bv_pos;
    nodes[5 * v + 1] = d.bv_pos_rank;
    nodes[5 * v + 2] = d.parent;
    nodes[5 * v + 3] = d.child[0];
    nodes[5 * v + 4] = d.child[1];
  }
  for (uint32_t c = 0; c < 256; ++c) {
    leaves[c] = w->m_tree.m_c_to_leaf[c];
    paths[c] = w->m_tree.m_path[c];
  }
}

// select_support_mcl<t_b> of m_bv in the flat layout: info[8] as the other
// shims (size, arg_cnt, logn, logn4, nsb, has_long, sb words, pool words);
// with buffers, the words
void ref_huff_select(void* h, int t_b, uint64_t* info, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  const huff_t* w = (const huff_t*)h;
  auto go = [&](const auto& ss) {
    const uint64_t nsb = (ss.m_arg_cnt + 4095) >> 12;
    auto is_long = [&](uint64_t i) { return ss.m_longsuperblock != nullptr && !ss.m_longsuperblock[i].empty(); };
    auto words_of = [](const sdsl::int_vector<0>& v) { return (v.bit_size() + 63) >> 6; };
    uint64_t pw = 0;
    for (uint64_t i = 0; i < nsb; ++i) pw += words_of(is_long(i) ? ss.m_longsuperblock[i] : ss.m_miniblock[i]);
    info[0] = w->m_bv.bit_size();
    info[1] = ss.m_arg_cnt;
    info[2] = ss.m_logn;
    info[3] = ss.m_logn4;
    info[4] = nsb;
    info[5] = ss.m_longsuperblock != nullptr;
    info[6] = ss.m_arg_cnt ? words_of(ss.m_superblock) : 0;
    info[7] = pw;
    if (!sb_words || !ss.m_arg_cnt) return;
    memcpy(sb_words, ss.m_superblock.data(), words_of(ss.m_superblock) * 8);
    uint64_t off = 0;
    for (uint64_t i = 0; i < nsb; ++i) {
      const sdsl::int_vector<0>& b = is_long(i) ? ss.m_longsuperblock[i] : ss.m_miniblock[i];
      desc[i] = (off << 8) | ((uint64_t)is_long(i) << 7) | b.width();
      memcpy(pool + off, b.data(), words_of(b) * 8);
      off += words_of(b);
    }
  };
  if (t_b) go(w->m_bv_select1);
  else go(w->m_bv_select0);
}

uint64_t ref_huff_access(void* h, uint64_t i) { return (*(const huff_t*)h)[i]; }
uint64_t ref_huff_rank_query(void* h, uint64_t i, uint64_t c) { return ((const huff_t*)h)->rank(i, (uint8_t)c); }
uint64_t ref_huff_select_query(void* h, uint64_t i, uint64_t c) { return ((const huff_t*)h)->select(i, (uint8_t)c); }
void ref_huff_inverse_select(void* h, uint64_t i, uint64_t* out) {
  auto r = ((const huff_t*)h)->inverse_select(i);
  out[0] = r.first;
  out[1] = r.second;
}
}
