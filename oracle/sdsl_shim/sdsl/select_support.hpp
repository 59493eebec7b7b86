// Minimal stand-in for sdsl-lite's select_support.hpp (TEST INFRASTRUCTURE
// ONLY; see int_vector.hpp in this directory).  Restates the base class (with
// its `vv` alias of the supported vector) and the single-bit select traits:
// for pattern `1` the args are set bits, for pattern `0` the set bits of the
// complement; the "first word" variants ignore bits below `offset`; sel()
// returns the in-word position of the i-th arg.
#ifndef WTG_SDSL_SHIM_SELECT_SUPPORT
#define WTG_SDSL_SHIM_SELECT_SUPPORT
#include "int_vector.hpp"
#include "util.hpp"

namespace sdsl {

class select_support {
 protected:
  const bit_vector* m_v;

 public:
  typedef bit_vector::size_type size_type;
  const bit_vector*& vv;
  explicit select_support(const bit_vector* v = nullptr) : m_v(v), vv(m_v) {}
  select_support(const select_support& o) : m_v(o.m_v), vv(m_v) {}
  virtual ~select_support() {}
};

template <uint8_t t_b, uint8_t t_pat_len>
struct select_support_trait;

template <>
struct select_support_trait<1, 1> {
  typedef uint64_t size_type;
  static size_type arg_cnt(const bit_vector& v) { return util::cnt_one_bits(v); }
  static size_type args_in_the_first_word(uint64_t w, uint8_t offset, uint64_t) {
    return bits::cnt(w & bits::lo_unset_f(offset));
  }
  static size_type ith_arg_pos_in_the_first_word(uint64_t w, size_type i, uint8_t offset, uint64_t) {
    return bits::sel(w & bits::lo_unset_f(offset), (uint32_t)i);
  }
  static size_type args_in_the_word(uint64_t w, uint64_t&) { return bits::cnt(w); }
  static size_type ith_arg_pos_in_the_word(uint64_t w, size_type i, uint64_t) {
    return bits::sel(w, (uint32_t)i);
  }
  static bool found_arg(size_type i, const bit_vector& v) { return v[i]; }
  static uint64_t init_carry(const uint64_t*, size_type) { return 0; }
  static uint64_t get_carry(uint64_t) { return 0; }
};

template <>
struct select_support_trait<0, 1> {
  typedef uint64_t size_type;
  static size_type arg_cnt(const bit_vector& v) { return v.bit_size() - util::cnt_one_bits(v); }
  static size_type args_in_the_first_word(uint64_t w, uint8_t offset, uint64_t) {
    return bits::cnt((~w) & bits::lo_unset_f(offset));
  }
  static size_type ith_arg_pos_in_the_first_word(uint64_t w, size_type i, uint8_t offset, uint64_t) {
    return bits::sel((~w) & bits::lo_unset_f(offset), (uint32_t)i);
  }
  static size_type args_in_the_word(uint64_t w, uint64_t&) { return bits::cnt(~w); }
  static size_type ith_arg_pos_in_the_word(uint64_t w, size_type i, uint64_t) {
    return bits::sel(~w, (uint32_t)i);
  }
  static bool found_arg(size_type i, const bit_vector& v) { return !v[i]; }
  static uint64_t init_carry(const uint64_t*, size_type) { return 0; }
  static uint64_t get_carry(uint64_t) { return 0; }
};

}  // namespace sdsl
#endif
