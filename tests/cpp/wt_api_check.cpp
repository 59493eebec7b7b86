// Drives the reference-shaped C++ interface (host/wtg_reference_api.hpp) the
// way levelWT/WTTime.C and a wt_int user do, and writes what it got so the
// Python test can compare it with the oracle.
//   wt_api_check <symbols.bin> <n> <sigma> <out.bin>
// out.bin: 2*sigma WTnode records, then the WT() bitvector words, then the
// rank_support_v table over those words, then three u64 checks (wt_int access
// mismatches, sum over c of rank(n, c) minus n, select_support_mcl<1> arg_cnt),
// then the range queries of 64 fixed queries q (i = q*n/64, j = i + n/8 capped
// at n, c = s[i] or 0): per q lex_count (3), lex_smaller_count (2),
// range_search_2d(i, j-1, c/2, c) count and its points' position sum (2),
// interval_symbols k and sum of its symbols (2), then four u64 checks of the
// root's expand (left size + right size - n, left.level, right.sym, and the
// expanded range sizes minus the range size).  The sdsl serialize() streams of
// the wt_int, the rank_support_v and the select_support_mcl<1> go to
// out.bin.wt_int, out.bin.rank and out.bin.sel1 (wtg::store_to_file).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
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

  std::vector<uint64_t> rq;
  std::vector<uint64_t> cs(sigma + 1), ri(sigma + 1), rj(sigma + 1);
  for (uint64_t q = 0; q < 64; ++q) {
    const uint64_t i = q * (uint64_t)n / 64, j = std::min<uint64_t>(n, i + n / 8 + 1);
    const uint64_t c = i < n ? (uint64_t)s[i] : 0;
    auto lc = wt.lex_count(i, j, c);
    rq.push_back(std::get<0>(lc));
    rq.push_back(std::get<1>(lc));
    rq.push_back(std::get<2>(lc));
    auto ls = wt.lex_smaller_count(i, c);
    rq.push_back(std::get<0>(ls));
    rq.push_back(std::get<1>(ls));
    auto r2 = wt.range_search_2d(i, j - 1, c / 2, c);
    uint64_t psum = 0;
    for (auto& p : r2.second) psum += p.first;
    rq.push_back(r2.first);
    rq.push_back(psum);
    uint64_t k = 0, csum = 0;
    wt.interval_symbols(i, j, k, cs, ri, rj);
    for (uint64_t t = 0; t < k; ++t) csum += cs[t];
    rq.push_back(k);
    rq.push_back(csum);
  }
  auto kids = wt.expand(wt.root());
  auto rr = wt.expand(wt.root(), wtg::wt_int::range_type(n / 4, n / 2));
  const uint64_t rsz = (rr.first.second - rr.first.first + 1) + (rr.second.second - rr.second.first + 1);
  rq.push_back(kids.first.size + kids.second.size - n);
  rq.push_back(kids.first.level);
  rq.push_back(kids.second.sym);
  rq.push_back(rsz - (n / 2 - n / 4 + 1));

  FILE* o = std::fopen(argv[4], "wb");
  if (!o) return 4;
  std::fwrite(r.first, sizeof(WTnode), 2 * (size_t)sigma, o);
  std::fwrite(r.second, sizeof(long), nw, o);
  std::fwrite(rank.data(), sizeof(uint64_t), rank.size(), o);
  const uint64_t checks[3] = {bad, total - n, ss.arg_cnt()};
  std::fwrite(checks, sizeof(uint64_t), 3, o);
  std::fwrite(rq.data(), sizeof(uint64_t), rq.size(), o);
  std::fclose(o);
  // sdsl streams, as store_to_file writes them: <out>.wt_int, .rank, .sel1
  const std::string base(argv[4]);
  if (!wtg::store_to_file(wt, base + ".wt_int") || !wtg::store_to_file(rs, base + ".rank") ||
      !wtg::store_to_file(ss, base + ".sel1"))
    return 5;
  std::free(r.first);
  std::free(r.second);
  return 0;
}
