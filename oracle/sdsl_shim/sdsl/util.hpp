// Minimal stand-in for sdsl-lite's util.hpp (TEST INFRASTRUCTURE ONLY; see
// int_vector.hpp in this directory for why it exists).
#ifndef WTG_SDSL_SHIM_UTIL
#define WTG_SDSL_SHIM_UTIL
#include <sstream>
#include <string>
#include <typeinfo>
#include <utility>
#include "int_vector.hpp"

namespace sdsl {
namespace util {
template <class T>
std::string class_name(const T&) { return typeid(T).name(); }
template <class T>
std::string to_string(const T& t) {
  std::ostringstream s;
  s << t;
  return s.str();
}
// number of set bits in the data words of v (bits past the end are zero)
template <class V>
uint64_t cnt_one_bits(const V& v) {
  uint64_t r = 0;
  const uint64_t* d = v.data();
  for (uint64_t i = 0; i < (v.capacity() >> 6); ++i) r += bits::cnt(d[i]);
  return r;
}
template <class S, class V>
void init_support(S& s, const V* v) {
  S tmp(v);
  s = std::move(tmp);
  s.set_vector(v);
}
template <class S, class V>
void swap_support(S& s1, S& s2, const V* v1, const V* v2) {
  std::swap(s1, s2);
  s1.set_vector(v1);
  s2.set_vector(v2);
}
}  // namespace util
}  // namespace sdsl
#endif
