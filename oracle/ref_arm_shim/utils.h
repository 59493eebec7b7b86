// Portable stand-in for the reference's utils.h (PBBS helpers), used only to
// build the reference's own levelWT / rank / select code as the timed CPU
// baseline on hosts where its x86 inline assembly (lock cmpxchg, lock xadd)
// does not assemble, such as aarch64.
//
// TEST AND BENCHMARK INFRASTRUCTURE ONLY.  The reference's sources include
// "utils.h" by name; oracle/Makefile's bench-ref target compiles them from a
// staged copy that leaves utils.h out, so this directory's file is found
// through the include path instead.  It provides the names those sources
// use -- newA, utils::log2Up, utils::CAS, utils::addF, utils::identityF --
// with the same meaning: log2Up(i) is the number of bits of i - 1 (log2
// rounded up), CAS is an atomic compare-and-swap of a 4- or 8-byte value
// returning whether it swapped, addF/identityF are the sum and identity
// functors.
#ifndef _BENCH_UTILS_INCLUDED
#define _BENCH_UTILS_INCLUDED
#include <algorithm>
#include <cstdlib>
#include <iostream>
#include "parallel.h"

#define newA(T, count) (T*)malloc((count) * sizeof(T))

namespace utils {

template <class T>
static int log2Up(T i) {
  int bits = 0;
  for (T b = i - 1; b > 0; b = b >> 1) ++bits;
  return bits;
}

template <class ET>
inline bool CAS(ET* ptr, ET oldv, ET newv) {
  static_assert(sizeof(ET) == 4 || sizeof(ET) == 8, "CAS on 4 or 8 bytes");
  return __atomic_compare_exchange(ptr, &oldv, &newv, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
}

template <class E>
struct identityF {
  E operator()(const E& x) { return x; }
};

template <class E>
struct addF {
  E operator()(const E& a, const E& b) const { return a + b; }
};

}  // namespace utils
#endif
