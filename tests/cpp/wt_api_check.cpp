// Drives the reference-shaped C++ interface (host/wtg_reference_api.hpp) the
// way levelWT/WTTime.C and a wt_int user do, and writes what it got so the
// Python test can compare it with the oracle.
//   wt_api_check <symbols.bin> <n> <sigma> <out.bin>
// out.bin: 2*sigma WTnode records, then the WT() bitvector words, then the
// rank_support_v table over those words, then three u64 checks (wt_int access
// mismatches, sum over c of rank(n, c) minus n, select_support_mcl<1> arg_cnt).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../wavelet-suffix-fm-index_gb300/host/wtg_reference_api.hpp"

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s symbols.bin n sigma out.bin\n", argv[0]);
    return 2;
  }
  const uintT n = (uintT)std::strtoull(argv[2], nullptr, 10);
  const uintT sigma = (uintT)std::strtoull(argv[3], nullptr, 10);
  std::vector<symbol> s(n);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(s.data(), sizeof(symbol), n, f) != n) return 3;
  std::fclose(f);

  std::pair<WTnode*, long*> r = WT(s.data(), n, sigma);
  const int levels = wtg::levels_for_sigma(sigma);
  const uint64_t nbits = (uint64_t)n * levels, nw = (nbits + 63) / 64;

  std::vector<uint64_t> words(nw + 1, 0);  // one spare word, as int_vector keeps
  for (uint64_t i = 0; i < nw; ++i) words[i] = (uint64_t)r.second[i];
  wtg::rank_support_v rs(words.data(), nbits);
  std::vector<uint64_t> rank = rs.basic_block();
  wtg::select_support_mcl<1> ss(words.data(), nbits);

  wtg::wt_int wt(s, n, (uint32_t)levels);
  uint64_t bad = 0, total = 0;
  for (uintT i = 0; i < n; ++i) bad += wt[i] != (uint64_t)s[i];
  for (uintT c = 0; c < sigma; ++c) total += wt.rank(n, c);

  FILE* o = std::fopen(argv[4], "wb");
  if (!o) return 4;
  std::fwrite(r.first, sizeof(WTnode), 2 * (size_t)sigma, o);
  std::fwrite(r.second, sizeof(long), nw, o);
  std::fwrite(rank.data(), sizeof(uint64_t), rank.size(), o);
  const uint64_t checks[3] = {bad, total - n, ss.arg_cnt()};
  std::fwrite(checks, sizeof(uint64_t), 3, o);
  std::fclose(o);
  std::free(r.first);
  std::free(r.second);
  return 0;
}
