// ref_levelwt_shim.cpp -- exposes the reference's own WT() builder over a C ABI
// so the tests can pin the oracle against it.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the unmodified reference sources (wavelet/levelWT/WT.C, or serialWT/WT.C)
// found under the read-only reference checkout, with the reference directory on
// the include path; the result goes to oracle/_ref/ and is never shipped.
// The symbol and index widths follow the reference's own compile-time knobs:
// -DINT makes symbols uintT, -DLONG makes uintT 64-bit (wavelet/levelWT/WT.h:24-43,
// parallel.h:71-81).
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>
#include "parallel.h"
#include "utils.h"
#include "WT.h"

extern "C" {

// Width in bytes of the reference's symbol and uintT types in this build.
int ref_symbol_bytes(void) { return (int)sizeof(symbol); }
int ref_uint_bytes(void) { return (int)sizeof(uintT); }

// Calls WT(s, n, sigma) and copies its outputs: `words` receives
// ceil(n*levels/64) words; `nodes` receives 2*sigma WTnode records in the
// reference's own struct layout (5 x uintT).  Node records the reference never
// writes hold whatever malloc returned; callers compare reachable nodes only.
int ref_wt(const void* s, uint64_t n, uint64_t sigma, uint64_t* words, uint64_t nwords,
           void* nodes) {
  symbol* in = (symbol*)malloc(sizeof(symbol) * (n ? n : 1));
  if (!in) return -1;
  memcpy(in, s, sizeof(symbol) * n);
  std::pair<WTnode*, long*> R = WT(in, (uintT)n, (uintT)sigma);
  memcpy(words, R.second, nwords * sizeof(uint64_t));
  if (nodes) memcpy(nodes, R.first, 2 * sigma * sizeof(WTnode));
  free(R.first);
  free(R.second);
  free(in);
  return 0;
}

// Seconds of WT(text, n_t, sigma) over T texts laid end to end (offs[t] ..
// offs[t + 1]), the texts spread over the OpenMP threads (each WT() call
// then runs on its thread: the reference's own parallel_for inside it is a
// nested region).  Inputs are copied to per-text buffers before the clock
// starts and the outputs freed after it stops.  < 0 when memory runs out.
double ref_wt_batch_time(const uint8_t* concat, const uint64_t* offs, uint64_t T, uint64_t sigma) {
  std::vector<symbol*> in(T, nullptr);
  std::vector<std::pair<WTnode*, long*>> out(T);
  bool ok = true;
  for (uint64_t t = 0; t < T; ++t) {
    const uint64_t n = offs[t + 1] - offs[t];
    in[t] = (symbol*)malloc(sizeof(symbol) * (n ? n : 1));
    if (!in[t]) ok = false;
    else for (uint64_t i = 0; i < n; ++i) in[t][i] = (symbol)concat[offs[t] + i];
  }
  double secs = -1.0;
  if (ok) {
    const auto t0 = std::chrono::steady_clock::now();
#if defined(OPENMP)
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long t = 0; t < (long)T; ++t) out[t] = WT(in[t], (uintT)(offs[t + 1] - offs[t]), (uintT)sigma);
    const auto t1 = std::chrono::steady_clock::now();
    secs = std::chrono::duration<double>(t1 - t0).count();
    for (uint64_t t = 0; t < T; ++t) {
      free(out[t].first);
      free(out[t].second);
    }
  }
  for (uint64_t t = 0; t < T; ++t) free(in[t]);
  return secs;
}

// Seconds of one WT(s, n, sigma) call -- the timed CPU baseline.  The input
// (n symbols of in_bytes bytes) is widened to the build's symbol type before
// the clock starts; the outputs are freed after it stops.  Returns < 0 when
// memory runs out.
double ref_wt_time(const void* s, int in_bytes, uint64_t n, uint64_t sigma) {
  symbol* in = (symbol*)malloc(sizeof(symbol) * (n ? n : 1));
  if (!in) return -1.0;
  for (uint64_t i = 0; i < n; ++i)
    in[i] = in_bytes == 1 ? (symbol)((const uint8_t*)s)[i]
            : in_bytes == 4 ? (symbol)((const uint32_t*)s)[i] : (symbol)((const uint64_t*)s)[i];
  const auto t0 = std::chrono::steady_clock::now();
  std::pair<WTnode*, long*> R = WT(in, (uintT)n, (uintT)sigma);
  const auto t1 = std::chrono::steady_clock::now();
  free(R.first);
  free(R.second);
  free(in);
  return std::chrono::duration<double>(t1 - t0).count();
}
}
