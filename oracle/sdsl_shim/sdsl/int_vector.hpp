// Minimal stand-in for the parts of sdsl-lite's int_vector.hpp that the
// reference's rank_support_v_par.hpp and select_support_mcl_par.hpp use.
//
// TEST INFRASTRUCTURE ONLY.  sdsl-lite is not vendored in the reference tree
// and is not installed here, so this header restates the documented
// behaviour of the few sdsl types those headers touch, to let the reference's
// own rank/select construction code compile and run as the pin for the
// oracle.  Semantics restated:
//   * int_vector<w> stores size() entries of width w bits packed LSB-first in
//     64-bit words; the bit size is size()*w; capacity() is the bit size
//     rounded up to a multiple of 64; one extra zero word follows the data
//     (sdsl allocates it, and rank_support_v's constructor reads it when the
//     capacity is a multiple of 512).
//   * int_vector<0> has its width chosen at run time (default 64).
//   * int_vector<64>::operator[] yields a real uint64_t&.
//   * serialize() writes the size in bits as a uint64, then -- for the
//     run-time width int_vector<0> only -- the width as one byte, then the
//     ceil(bits/64) data words; load() reads the same stream.
#ifndef WTG_SDSL_SHIM_INT_VECTOR
#define WTG_SDSL_SHIM_INT_VECTOR
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <istream>
#include <ostream>
#include <string>
#include <type_traits>
#include <utility>

namespace sdsl {

struct structure_tree_node {};
struct structure_tree {
  static structure_tree_node* add_child(structure_tree_node*, const std::string&, const std::string&) {
    return nullptr;
  }
  static void add_size(structure_tree_node*, uint64_t) {}
};

namespace bits {
inline uint32_t hi(uint64_t x) { return x == 0 ? 0u : 63u - (uint32_t)__builtin_clzll(x); }
inline uint32_t cnt(uint64_t x) { return (uint32_t)__builtin_popcountll(x); }
// position of the i-th (1-based) set bit
inline uint32_t sel(uint64_t x, uint32_t i) {
  for (uint32_t k = 1; k < i; ++k) x &= x - 1;
  return (uint32_t)__builtin_ctzll(x);
}
inline uint64_t lo_set_f(uint32_t k) { return k >= 64 ? ~0ull : ((1ull << k) - 1); }
// x with its 64 bits in reverse order
inline uint64_t rev(uint64_t x) {
  uint64_t r = 0;
  for (int k = 0; k < 64; ++k, x >>= 1) r = (r << 1) | (x & 1);
  return r;
}
inline uint64_t lo_unset_f(uint32_t k) { return k >= 64 ? 0ull : (~0ull << k); }
}  // namespace bits

template <uint8_t t_width>
class int_vector;

template <uint8_t t_width>
class int_vector_reference {
  int_vector<t_width>* m_v;
  uint64_t m_i;

 public:
  int_vector_reference(int_vector<t_width>* v, uint64_t i) : m_v(v), m_i(i) {}
  operator uint64_t() const { return m_v->get(m_i); }
  int_vector_reference& operator=(uint64_t x) {
    m_v->set(m_i, x);
    return *this;
  }
  int_vector_reference& operator=(const int_vector_reference& r) { return *this = (uint64_t)r; }
};

template <uint8_t t_width = 0>
class int_vector {
 public:
  typedef uint64_t value_type;
  typedef uint64_t size_type;
  typedef int64_t difference_type;
  typedef typename std::conditional<t_width == 64, uint64_t&, int_vector_reference<t_width>>::type reference;

  uint64_t m_size = 0;  // bits
  uint64_t* m_data = nullptr;
  uint8_t m_width = t_width ? t_width : 64;

  explicit int_vector(size_type size = 0, value_type default_value = 0,
                      uint8_t width = t_width ? t_width : 64) {
    m_width = t_width ? t_width : width;
    alloc(size * m_width);
    if (default_value)
      for (size_type i = 0; i < size; ++i) set(i, default_value);
  }
  int_vector(const int_vector& o) : m_width(o.m_width) {
    alloc(o.m_size);
    memcpy(m_data, o.m_data, words_alloc(o.m_size) * 8);
  }
  int_vector(int_vector&& o) noexcept : m_size(o.m_size), m_data(o.m_data), m_width(o.m_width) {
    o.m_data = nullptr;
    o.m_size = 0;
  }
  int_vector& operator=(const int_vector& o) {
    if (this != &o) {
      free(m_data);
      m_width = o.m_width;
      alloc(o.m_size);
      memcpy(m_data, o.m_data, words_alloc(o.m_size) * 8);
    }
    return *this;
  }
  int_vector& operator=(int_vector&& o) noexcept {
    if (this != &o) {
      free(m_data);
      m_size = o.m_size;
      m_data = o.m_data;
      m_width = o.m_width;
      o.m_data = nullptr;
      o.m_size = 0;
    }
    return *this;
  }
  ~int_vector() { free(m_data); }

  static uint64_t words_alloc(uint64_t bits) { return ((bits + 63) >> 6) + 1; }
  void alloc(uint64_t bits) {
    m_size = bits;
    m_data = (uint64_t*)calloc(words_alloc(bits), 8);
  }

  size_type size() const { return m_size / m_width; }
  size_type bit_size() const { return m_size; }
  size_type capacity() const { return ((m_size + 63) >> 6) << 6; }
  bool empty() const { return m_size == 0; }
  uint8_t width() const { return m_width; }
  uint64_t* data() { return m_data; }
  const uint64_t* data() const { return m_data; }

  void resize(size_type n) {
    uint64_t bits = n * m_width;
    uint64_t* d = (uint64_t*)calloc(words_alloc(bits), 8);
    if (m_data) {
      uint64_t keep = words_alloc(bits) < words_alloc(m_size) ? words_alloc(bits) : words_alloc(m_size);
      memcpy(d, m_data, keep * 8);
      free(m_data);
    }
    m_data = d;
    m_size = bits;
    // keep the bits past the end zero
    if (bits & 63) m_data[bits >> 6] &= bits::lo_set_f((uint32_t)(bits & 63));
    for (uint64_t w = (bits + 63) >> 6; w < words_alloc(bits); ++w) m_data[w] = 0;
  }

  uint64_t get(size_type i) const {
    uint64_t off = i * m_width;
    uint64_t wi = off >> 6;
    uint32_t sh = (uint32_t)(off & 63);
    uint64_t v = m_data[wi] >> sh;
    if (sh + m_width > 64) v |= m_data[wi + 1] << (64 - sh);
    return v & bits::lo_set_f(m_width);
  }
  void set(size_type i, uint64_t x) {
    uint64_t off = i * m_width;
    uint64_t wi = off >> 6;
    uint32_t sh = (uint32_t)(off & 63);
    uint64_t mask = bits::lo_set_f(m_width);
    x &= mask;
    m_data[wi] = (m_data[wi] & ~(mask << sh)) | (x << sh);
    if (sh + m_width > 64) {
      uint32_t r = 64 - sh;
      m_data[wi + 1] = (m_data[wi + 1] & ~(mask >> r)) | (x >> r);
    }
  }

  // the `len` (<= 64) low bits of x at bit position idx
  void set_int(size_type idx, uint64_t x, uint8_t len = 64) {
    for (uint8_t k = 0; k < len; ++k) {
      const uint64_t p = idx + k;
      const uint64_t m = 1ull << (p & 63);
      m_data[p >> 6] = ((x >> k) & 1) ? (m_data[p >> 6] | m) : (m_data[p >> 6] & ~m);
    }
  }

  reference operator[](size_type i) {
    if constexpr (t_width == 64) return m_data[i];
    else return int_vector_reference<t_width>(this, i);
  }
  value_type operator[](size_type i) const { return get(i); }

  void swap(int_vector& o) {
    std::swap(m_size, o.m_size);
    std::swap(m_data, o.m_data);
    std::swap(m_width, o.m_width);
  }

  size_type serialize(std::ostream& out, structure_tree_node* = nullptr, std::string = "") const {
    const uint64_t bits = m_size;
    out.write(reinterpret_cast<const char*>(&bits), sizeof(bits));
    size_type written = sizeof(bits);
    if (t_width == 0) {
      const uint8_t w = m_width;
      out.write(reinterpret_cast<const char*>(&w), 1);
      written += 1;
    }
    const uint64_t nw = (bits + 63) >> 6;
    if (nw) out.write(reinterpret_cast<const char*>(m_data), (std::streamsize)(nw * 8));
    return written + nw * 8;
  }
  void load(std::istream& in) {
    uint64_t bits = 0;
    in.read(reinterpret_cast<char*>(&bits), sizeof(bits));
    if (t_width == 0) {
      uint8_t w = 64;
      in.read(reinterpret_cast<char*>(&w), 1);
      m_width = w;
    }
    free(m_data);
    alloc(bits);
    const uint64_t nw = (bits + 63) >> 6;
    if (nw) in.read(reinterpret_cast<char*>(m_data), (std::streamsize)(nw * 8));
  }
};

typedef int_vector<1> bit_vector;

}  // namespace sdsl
#endif
