// Portable stand-in for <immintrin.h> where the reference's sequence.h
// includes it for _popcnt64 (TEST AND BENCHMARK INFRASTRUCTURE ONLY; found
// first through the include path of oracle/Makefile's bench-ref target).
#pragma once
#include <cstdint>
static inline long long _popcnt64(unsigned long long x) { return __builtin_popcountll(x); }
