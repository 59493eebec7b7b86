// Minimal stand-in for sdsl-lite's rank_support.hpp (TEST INFRASTRUCTURE ONLY;
// see int_vector.hpp in this directory).  Restates the base class and the
// single-bit rank traits: pattern `1` counts set bits of each word, pattern
// `0` counts set bits of its complement; word_rank counts them below idx%64.
#ifndef WTG_SDSL_SHIM_RANK_SUPPORT
#define WTG_SDSL_SHIM_RANK_SUPPORT
#include "int_vector.hpp"
#include "util.hpp"

namespace sdsl {

class rank_support {
 protected:
  const bit_vector* m_v = nullptr;

 public:
  typedef bit_vector::size_type size_type;
  explicit rank_support(const bit_vector* v = nullptr) : m_v(v) {}
  virtual ~rank_support() {}
};

template <uint8_t t_b, uint8_t t_pat_len>
struct rank_support_trait;

template <>
struct rank_support_trait<1, 1> {
  typedef uint64_t size_type;
  static size_type init_carry() { return 0; }
  static size_type args_in_the_word(uint64_t w, uint64_t&) { return bits::cnt(w); }
  static uint32_t word_rank(const uint64_t* data, size_type idx) {
    return bits::cnt(data[idx >> 6] & bits::lo_set_f((uint32_t)(idx & 0x3F)));
  }
};

template <>
struct rank_support_trait<0, 1> {
  typedef uint64_t size_type;
  static size_type init_carry() { return 0; }
  static size_type args_in_the_word(uint64_t w, uint64_t&) { return bits::cnt(~w); }
  static uint32_t word_rank(const uint64_t* data, size_type idx) {
    return bits::cnt((~data[idx >> 6]) & bits::lo_set_f((uint32_t)(idx & 0x3F)));
  }
};

}  // namespace sdsl
#endif
