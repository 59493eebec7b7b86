// Minimal stand-in for sdsl-lite's wt_helper.hpp and the iterator / buffer
// names wt_int's declarations mention (TEST INFRASTRUCTURE ONLY; see
// int_vector.hpp in this directory).  Restated: the names, the range types
// (a range is a closed interval [first, second] of positions), the raw-bytes
// member I/O, the character counting helpers and the byte alphabet's
// prefix-code tree in breadth-first layout that wt_pc uses.
#ifndef WTG_SDSL_SHIM_WT_HELPER
#define WTG_SDSL_SHIM_WT_HELPER
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include "int_vector.hpp"
#include "sdsl_concepts.hpp"

namespace sdsl {
typedef std::pair<uint64_t, uint64_t> range_type;
typedef std::vector<range_type> range_vec_type;

template <class t_rac>
class random_access_const_iterator {
 public:
  random_access_const_iterator(const t_rac*, uint64_t) {}
};

template <uint8_t t_width = 0>
class int_vector_buffer {
 public:
  uint64_t size() const { return 0; }
  uint8_t width() const { return 64; }
  std::string filename() const { return std::string(); }
  uint64_t operator[](uint64_t) const { return 0; }
};

inline std::string tmp_file(const std::string& f, const std::string& s) { return f + s; }
inline int remove(const std::string&) { return 0; }
template <class T>
bool load_from_file(T&, const std::string&) { return false; }
// ---- prefix-code trees (what wt_pc and its shapes use)
//
// A node of a code tree as a shape builds it: frequency, symbol (of a leaf),
// parent and children (undef where absent).
struct pc_node {
  uint64_t freq;
  uint64_t sym;
  uint64_t parent;
  uint64_t child[2];
  enum : uint64_t { undef = 0xFFFFFFFFFFFFFFFFull };
  pc_node(uint64_t f = 0, uint64_t s = 0, uint64_t p = undef, uint64_t c0 = undef, uint64_t c1 = undef)
      : freq(f), sym(s), parent(p) {
    child[0] = c0;
    child[1] = c1;
  }
};

// The code tree over the byte alphabet in breadth-first order: the root is
// node 0 (the shape's last node), then the nodes in the order a first-in
// first-out traversal meets them, a node's left child (child[0]) before its
// right.  bv_pos(v) is where v's bitvector starts in the wavelet tree's
// concatenated bit_vector -- the sizes (frequencies) of the inner nodes met
// before v, added up; bv_size receives the total.  bv_pos_rank(v) is, for a
// leaf, its symbol, and for an inner node the ones before bv_pos(v)
// (init_node_ranks).  bit_path(c) is symbol c's path from the root, bit d set
// when the (d+1)-th edge goes to a right child, in the low 56 bits, and the
// path length in the top 8 bits (0 for a symbol not in the tree).
template <bool t_dfs_shape = false>
struct _byte_tree {
  typedef uint16_t node_type;
  typedef uint8_t value_type;
  typedef byte_alphabet_tag alphabet_category;
  enum : node_type { undef = 0xFFFF };
  enum : uint32_t { fixed_sigma = 256 };
  enum : uint8_t { int_width = 8 };
  struct tree_node {
    uint64_t bv_pos = 0;
    uint64_t bv_pos_rank = 0;
    node_type parent = undef;
    node_type child[2] = {undef, undef};
  };
  std::vector<tree_node> m_nodes;
  node_type m_c_to_leaf[fixed_sigma];
  uint64_t m_path[fixed_sigma];

  _byte_tree() {
    for (uint32_t c = 0; c < fixed_sigma; ++c) {
      m_c_to_leaf[c] = undef;
      m_path[c] = 0;
    }
  }
  template <class t_wt>
  _byte_tree(const std::vector<pc_node>& shape, uint64_t& bv_size, const t_wt*) : _byte_tree() {
    bv_size = 0;
    if (shape.empty()) return;
    m_nodes.resize(shape.size());
    std::vector<uint64_t> from(shape.size());  // breadth-first index -> shape index
    from[0] = shape.size() - 1;
    size_t placed = 1;
    for (size_t v = 0; v < placed; ++v) {  // the placed nodes form the queue
      const pc_node& sn = shape[from[v]];
      tree_node& tn = m_nodes[v];
      tn.bv_pos = bv_size;
      const bool inner = sn.child[0] != pc_node::undef;
      if (inner) {
        bv_size += sn.freq;
        for (int k = 0; k < 2; ++k) {
          from[placed] = sn.child[k];
          m_nodes[placed].parent = (node_type)v;
          tn.child[k] = (node_type)placed;
          ++placed;
        }
      } else {
        tn.bv_pos_rank = sn.sym;
        m_c_to_leaf[(uint8_t)sn.sym] = (node_type)v;
      }
    }
    for (uint32_t c = 0; c < fixed_sigma; ++c) {
      if (m_c_to_leaf[c] == undef) continue;
      uint64_t path = 0, len = 0;
      for (node_type v = m_c_to_leaf[c]; v != 0; v = m_nodes[v].parent) {
        path = (path << 1) | (m_nodes[m_nodes[v].parent].child[1] == v ? 1u : 0u);
        ++len;
      }
      if (len > 56) throw std::logic_error("code depth above 56");
      m_path[c] = path | (len << 56);
    }
  }
  uint64_t size() const { return m_nodes.size(); }
  node_type root() const { return 0; }
  bool is_leaf(node_type v) const { return m_nodes[v].child[0] == undef; }
  node_type child(node_type v, uint8_t i) const { return m_nodes[v].child[i]; }
  node_type parent(node_type v) const { return m_nodes[v].parent; }
  uint64_t bv_pos(node_type v) const { return m_nodes[v].bv_pos; }
  uint64_t bv_pos_rank(node_type v) const { return m_nodes[v].bv_pos_rank; }
  bool is_valid(node_type v) const { return v != undef; }
  node_type c_to_leaf(value_type c) const { return m_c_to_leaf[c]; }
  uint64_t bit_path(value_type c) const { return m_path[c]; }
  template <class t_rank>
  void init_node_ranks(const t_rank& rank) {
    for (uint64_t v = 0; v < m_nodes.size(); ++v)
      if (m_nodes[v].child[0] != undef) m_nodes[v].bv_pos_rank = rank.rank(m_nodes[v].bv_pos);
  }
  void swap(_byte_tree& o) {
    std::swap(m_nodes, o.m_nodes);
    for (uint32_t c = 0; c < fixed_sigma; ++c) {
      std::swap(m_c_to_leaf[c], o.m_c_to_leaf[c]);
      std::swap(m_path[c], o.m_path[c]);
    }
  }
};

template <bool t_dfs_shape = false>
struct byte_tree {
  template <class t_wt>
  using type = _byte_tree<t_dfs_shape>;
};

// C[c] = occurrences of c among the first `size` entries of `text` (C grows
// to the largest symbol + 1)
template <class t_text, class t_rac>
void calculate_character_occurences(t_text& text, uint64_t size, t_rac& C) {
  C = t_rac();
  for (uint64_t i = 0; i < size; ++i) {
    const uint64_t c = text[i];
    if (c >= C.size()) C.resize(c + 1, 0);
    ++C[c];
  }
}

// the number of symbols that occur
template <class t_rac, class t_sigma>
void calculate_effective_alphabet_size(const t_rac& C, t_sigma& sigma) {
  sigma = 0;
  for (const auto& x : C) sigma += x > 0 ? 1 : 0;
}

// write_member / read_member of a plain value: its sizeof(T) bytes as they
// lie in memory
template <class T>
uint64_t write_member(const T& t, std::ostream& out, structure_tree_node* = nullptr, std::string = "") {
  out.write(reinterpret_cast<const char*>(&t), sizeof(T));
  return sizeof(T);
}
template <class T>
void read_member(T& t, std::istream& in) {
  in.read(reinterpret_cast<char*>(&t), sizeof(T));
}
}  // namespace sdsl
#endif
