// wtg_range.cu -- wt_int's range queries on the GPU, batched: lex_count,
// lex_smaller_count, range_search_2d (count and report), interval_symbols,
// expand(v) and expand(v, ranges) (wt_int/wt_int_par.hpp:684-1048).
//
// Every query walks heap nodes of the tree; the node table (per heap node
// its bit offset and the ones before it) replaces the reference's per-level
// rank probes of the node start and end, so a level costs one rank probe
// per query bound.
#include <algorithm>

#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {

namespace {

constexpr int RQ_STACK = 32;  // DFS stack entries per query (at most L + 1 <= 25 live)

__device__ __forceinline__ int level_of(uint64_t h) { return 63 - __clzll((long long)(h + 1)); }

// lex_count (wt_int_par.hpp:715-745) and, with SMALLER_ONLY,
// lex_smaller_count (:758-782): descend along c's path carrying the
// position bounds; symbols below / above c are counted where the path turns.
template <bool SMALLER_ONLY>
__global__ void wt_lex_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                              const ulonglong2* __restrict__ tab, uint64_t n, int L, const uint64_t* __restrict__ qi,
                              const uint64_t* __restrict__ qj, const uint64_t* __restrict__ qc, uint64_t nq,
                              uint64_t* __restrict__ out_rank, uint64_t* __restrict__ out_smaller,
                              uint64_t* __restrict__ out_greater) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  uint64_t i = qi[k], j = SMALLER_ONLY ? 0 : qj[k];
  const uint64_t c = qc[k];
  const bool ok = SMALLER_ONLY ? i <= n : (i <= j && j <= n);
  if (!ok) {
    out_rank[k] = NONE64;
    out_smaller[k] = NONE64;
    if (!SMALLER_ONLY) out_greater[k] = NONE64;
    return;
  }
  if ((1ull << L) <= c) {  // c above every symbol of the tree
    out_rank[k] = 0;
    out_smaller[k] = SMALLER_ONLY ? i : j - i;
    if (!SMALLER_ONLY) out_greater[k] = 0;
    return;
  }
  uint64_t smaller = 0, greater = 0, h = 0;
  ulonglong2 nd = __ldg(tab);
  for (int lv = 0; lv < L && (!SMALLER_ONLY || i); ++lv) {
    const uint64_t bit = (c >> (L - 1 - lv)) & 1;
    const uint64_t child = 2 * h + 1 + bit;
    const ulonglong2 next = lv + 1 < L ? __ldg(tab + child) : nd;
    const uint64_t oi = rank1_dev(rt, tree, nd.x + i) - nd.y;
    const uint64_t oj = SMALLER_ONLY ? 0 : rank1_dev(rt, tree, nd.x + j) - nd.y;
    if (bit) {
      smaller += SMALLER_ONLY ? i - oi : (j - i) - (oj - oi);
      i = oi;
      j = oj;
    } else {
      if (!SMALLER_ONLY) greater += oj - oi;
      i -= oi;
      j -= oj;
    }
    h = child;
    nd = next;
  }
  out_rank[k] = i;
  out_smaller[k] = smaller;
  if (!SMALLER_ONLY) out_greater[k] = greater;
}

// Value bounds of range_search_2d (wt_int_par.hpp:805-809): vrb is clamped
// to 2^L and vlb > vrb gives no point.  The reference's descent reaches the
// leaf 2^L - 1 when vlb = vrb = 2^L, so vlb = 2^L reads as 2^L - 1.
__device__ __forceinline__ bool value_bounds(int L, uint64_t& vlb, uint64_t& vrb) {
  const uint64_t top = 1ull << L;
  if (vrb > top) vrb = top;
  if (vlb > vrb) return false;
  if (vlb == top) vlb = top - 1;
  if (vrb == top) vrb = top - 1;
  return true;
}

struct RqEntry {
  uint64_t h, lb, rb;  // heap node and a position range inside it
};

// range_search_2d(..., report = false) (wt_int_par.hpp:801-871): the number of
// positions in [lb, rb] whose value lies in [vlb, vrb].  A node whose value
// range lies inside [vlb, vrb] adds its whole range at once (the reference
// descends to its leaves, which hold the same positions), so at most two
// partially covered nodes per level are expanded.
__global__ void wt_range_count_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                      const ulonglong2* __restrict__ tab, uint64_t n, int L,
                                      const uint64_t* __restrict__ qlb, const uint64_t* __restrict__ qrb,
                                      const uint64_t* __restrict__ qvlb, const uint64_t* __restrict__ qvrb,
                                      uint64_t nq, uint64_t* __restrict__ out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  const uint64_t lb0 = qlb[k], rb0 = qrb[k];
  uint64_t vlb = qvlb[k], vrb = qvrb[k];
  if (lb0 <= rb0 && rb0 >= n) {
    out[k] = NONE64;
    return;
  }
  if (lb0 > rb0 || !value_bounds(L, vlb, vrb)) {
    out[k] = 0;
    return;
  }
  RqEntry st[RQ_STACK];
  int sp = 0;
  st[sp++] = {0, lb0, rb0};
  uint64_t cnt = 0;
  bool overflow = false;
  while (sp) {
    const RqEntry e = st[--sp];
    const int lv = level_of(e.h);
    const uint64_t width = 1ull << (L - lv);
    const uint64_t ilb = (e.h + 1 - (1ull << lv)) << (L - lv);
    if (vlb <= ilb && ilb + width - 1 <= vrb) {
      cnt += e.rb - e.lb + 1;
      continue;
    }
    // partially covered, so an inner node: a pushed child's value range meets
    // [vlb, vrb], and a leaf that meets it lies inside it
    if (lv >= L) continue;
    const ulonglong2 nd = __ldg(tab + e.h);
    const uint64_t olb = rank1_dev(rt, tree, nd.x + e.lb) - nd.y;
    const uint64_t orb = rank1_dev(rt, tree, nd.x + e.rb + 1) - nd.y;
    const uint64_t zlb = e.lb - olb, zrb = e.rb + 1 - orb;
    const uint64_t mid = ilb + (width >> 1);
    if (sp + 2 > RQ_STACK) {
      overflow = true;
      break;
    }
    if (vlb < mid && zrb > zlb) st[sp++] = {2 * e.h + 1, zlb, zrb - 1};
    if (vrb >= mid && orb > olb) st[sp++] = {2 * e.h + 2, olb, orb - 1};
  }
  out[k] = overflow ? NONE64 : cnt;
}

// range_search_2d(..., report = true): warp per query.  The warp walks the
// tree depth first, left child first, down to every leaf that holds points
// (all lanes the same walk, so its probes are broadcasts); a leaf's points
// are split over the lanes, each climbing to its position with
// select1/select0 (wt_int_par.hpp:826-838).  Points go to
// pos/val[off[q] + t], t < off[q+1] - off[q], and below cap.
__global__ void wt_range_report_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                       const ulonglong2* __restrict__ tab, SelView s1, SelView s0, uint64_t n,
                                       int L, const uint64_t* __restrict__ qlb, const uint64_t* __restrict__ qrb,
                                       const uint64_t* __restrict__ qvlb, const uint64_t* __restrict__ qvrb,
                                       uint64_t nq, const uint64_t* __restrict__ off, uint64_t cap,
                                       uint64_t* __restrict__ pos, uint64_t* __restrict__ val) {
  const uint64_t q = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q >= nq) return;
  const uint64_t lb0 = qlb[q], rb0 = qrb[q];
  uint64_t vlb = qvlb[q], vrb = qvrb[q];
  if (lb0 > rb0 || rb0 >= n || !value_bounds(L, vlb, vrb)) return;
  const uint64_t base = off[q], lim = min(off[q + 1], cap);
  uint64_t emitted = 0;
  RqEntry st[RQ_STACK];
  int sp = 0;
  st[sp++] = {0, lb0, rb0};
  while (sp && base + emitted < lim) {
    const RqEntry e = st[--sp];
    const int lv = level_of(e.h);
    if (lv == L) {
      const uint64_t path = e.h + 1 - (1ull << L);
      const uint64_t cnt = e.rb - e.lb + 1;
      for (uint64_t t = lane; t < cnt && base + emitted + t < lim; t += 32) {
        uint64_t i = e.lb + t + 1;  // 1-based rank inside the leaf
        for (int kk = L; kk > 0; --kk) {
          const uint64_t hn = (1ull << (kk - 1)) - 1 + (path >> (L - kk + 1));  // node at level kk - 1
          const ulonglong2 nd = __ldg(tab + hn);
          if ((path >> (L - kk)) & 1) i = select_dev(s1, nd.y + i) - nd.x + 1;
          else i = select_dev(s0, nd.x - nd.y + i) - nd.x + 1;
        }
        pos[base + emitted + t] = i - 1;
        val[base + emitted + t] = path;
      }
      emitted += cnt;
      continue;
    }
    const uint64_t width = 1ull << (L - lv);
    const uint64_t ilb = (e.h + 1 - (1ull << lv)) << (L - lv);
    const ulonglong2 nd = __ldg(tab + e.h);
    const uint64_t olb = rank1_dev(rt, tree, nd.x + e.lb) - nd.y;
    const uint64_t orb = rank1_dev(rt, tree, nd.x + e.rb + 1) - nd.y;
    const uint64_t zlb = e.lb - olb, zrb = e.rb + 1 - orb;
    const uint64_t mid = ilb + (width >> 1);
    if (sp + 2 > RQ_STACK) break;  // not reached for L <= 24: a pop adds at most one live entry
    // right first, so the left child is expanded first
    if (vrb >= mid && orb > olb) st[sp++] = {2 * e.h + 2, olb, orb - 1};
    if (vlb < mid && zrb > zlb) st[sp++] = {2 * e.h + 1, zlb, zrb - 1};
  }
}

// interval_symbols (wt_int_par.hpp:684-702, recursion :119-158): the distinct
// symbols of [i, j) in increasing order with rank(i, c) and rank(j, c).
// Without FILL only their number; with FILL they go to off[q] + t,
// t < off[q+1] - off[q], and below cap.  Thread per query, depth first, left
// child first.
template <bool FILL>
__global__ void wt_interval_symbols_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                           const ulonglong2* __restrict__ tab, uint64_t n, int L,
                                           const uint64_t* __restrict__ qi, const uint64_t* __restrict__ qj,
                                           uint64_t nq, uint64_t* __restrict__ k_out,
                                           const uint64_t* __restrict__ off, uint64_t cap,
                                           uint64_t* __restrict__ cs, uint64_t* __restrict__ ri,
                                           uint64_t* __restrict__ rj) {
  const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t i0 = qi[q], j0 = qj[q];
  if (i0 > j0 || j0 > n) {
    if (!FILL) k_out[q] = NONE64;
    return;
  }
  uint64_t base = 0, lim = 0;
  if (FILL) {
    base = off[q];
    lim = min(off[q + 1], cap);
  }
  uint64_t k = 0;
  RqEntry st[RQ_STACK];  // (node, i, j) with i < j
  int sp = 0;
  if (i0 < j0) st[sp++] = {0, i0, j0};
  bool overflow = false;
  while (sp) {
    const RqEntry e = st[--sp];
    const int lv = level_of(e.h);
    if (lv == L) {
      if (FILL) {
        if (base + k >= lim) break;
        cs[base + k] = e.h + 1 - (1ull << L);
        ri[base + k] = e.lb;
        rj[base + k] = e.rb;
      }
      ++k;
      continue;
    }
    const ulonglong2 nd = __ldg(tab + e.h);
    const uint64_t oi = rank1_dev(rt, tree, nd.x + e.lb) - nd.y;
    const uint64_t oj = rank1_dev(rt, tree, nd.x + e.rb) - nd.y;
    if (sp + 2 > RQ_STACK) {
      overflow = true;
      break;
    }
    if (oj > oi) st[sp++] = {2 * e.h + 2, oi, oj};
    if ((e.rb - e.lb) > (oj - oi)) st[sp++] = {2 * e.h + 1, e.lb - oi, e.rb - oj};
  }
  if (!FILL) k_out[q] = overflow ? NONE64 : k;
}

// expand(v) (wt_int_par.hpp:966-984): v = (offset, size, level, sym) -> the
// left and right child in the same form; an invalid v (a leaf, or a range
// past the bits) gives UINT64_MAX fields
__global__ void wt_expand_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt, uint64_t n,
                                 int L, const uint64_t* __restrict__ nodes, uint64_t nn,
                                 uint64_t* __restrict__ left, uint64_t* __restrict__ right) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nn) return;
  const uint64_t off = nodes[4 * k], size = nodes[4 * k + 1], lv = nodes[4 * k + 2], sym = nodes[4 * k + 3];
  const uint64_t bits = (uint64_t)L * n;
  if (lv >= (uint64_t)L || off > bits || size > bits - off) {
    for (int f = 0; f < 4; ++f) left[4 * k + f] = right[4 * k + f] = NONE64;
    return;
  }
  const uint64_t ones = rank1_dev(rt, tree, off + size) - rank1_dev(rt, tree, off);
  const uint64_t lsize = size - ones;
  left[4 * k] = off + n;
  left[4 * k + 1] = lsize;
  left[4 * k + 2] = lv + 1;
  left[4 * k + 3] = sym << 1;
  right[4 * k] = off + n + lsize;
  right[4 * k + 1] = ones;
  right[4 * k + 2] = lv + 1;
  right[4 * k + 3] = (sym << 1) | 1;
}

// expand(v, ranges) (wt_int_par.hpp:1027-1048): closed ranges [s, e] of v
// mapped to its children, in unsigned 64-bit arithmetic as the reference
// (an empty range is e = s - 1); a range reaching past the bits gives
// UINT64_MAX bounds
__global__ void wt_expand_ranges_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                        uint64_t bits, uint64_t voff, const uint64_t* __restrict__ ranges,
                                        uint64_t nr, uint64_t* __restrict__ left, uint64_t* __restrict__ right) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nr) return;
  const uint64_t s = ranges[2 * k], e = ranges[2 * k + 1];
  const uint64_t p0 = voff + s, p1 = voff + e + 1;
  if (voff > bits || p0 > bits || p1 > bits) {
    left[2 * k] = left[2 * k + 1] = right[2 * k] = right[2 * k + 1] = NONE64;
    return;
  }
  const uint64_t v_sp_rank = rank1_dev(rt, tree, voff);
  const uint64_t sp_rank = rank1_dev(rt, tree, p0);
  const uint64_t right_size = rank1_dev(rt, tree, p1) - sp_rank;
  const uint64_t left_size = (e - s + 1) - right_size;
  const uint64_t right_sp = sp_rank - v_sp_rank, left_sp = s - right_sp;
  left[2 * k] = left_sp;
  left[2 * k + 1] = left_sp + left_size - 1;
  right[2 * k] = right_sp;
  right[2 * k + 1] = right_sp + right_size - 1;
}

// off[k] = count k (an invalid query's UINT64_MAX reads as 0), off[nq] = 0:
// the input of the exclusive scan that places each query's answers
__global__ void count_scan_input_kernel(const uint64_t* __restrict__ counts, uint64_t nq, uint64_t* __restrict__ off) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nq) off[k] = counts[k] == NONE64 ? 0 : counts[k];
  else if (k == nq) off[k] = 0;
}

unsigned qgrid(uint64_t threads) { return (unsigned)((threads + 255) / 256); }

int need_rank(const TreeImpl& t, const char* what) {
  if (!(t.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, std::string(what) + " needs a tree built with WTG_RANK");
  return WTG_OK;
}

}  // namespace

int answer_offsets(const uint64_t* counts, uint64_t nq, uint64_t* off, DevBuf& scratch, uint32_t* d_err,
                   cudaStream_t s) {
  count_scan_input_kernel<<<qgrid(nq + 1), 256, 0, s>>>(counts, nq, off);
  count_launch();
  WTG_CK(cudaGetLastError());
  return scan_exclusive_u64(off, off, nq + 1, scratch, d_err, s);
}

int launch_wt_lex_count(TreeImpl& t, const uint64_t* i, const uint64_t* j, const uint64_t* c, uint64_t nq,
                        uint64_t* rank_out, uint64_t* smaller_out, uint64_t* greater_out, cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "lex_count"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_lex_kernel<false><<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                                t.node_tab.as<ulonglong2>(), t.n, t.levels, i, j, c, nq, rank_out,
                                                smaller_out, greater_out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_lex_smaller_count(TreeImpl& t, const uint64_t* i, const uint64_t* c, uint64_t nq, uint64_t* rank_out,
                                uint64_t* smaller_out, cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "lex_smaller_count"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_lex_kernel<true><<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                               t.node_tab.as<ulonglong2>(), t.n, t.levels, i, nullptr, c, nq,
                                               rank_out, smaller_out, nullptr);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_range_count(TreeImpl& t, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                          const uint64_t* vrb, uint64_t nq, uint64_t* count_out, cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "range_search_2d"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_range_count_kernel<<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                                  t.node_tab.as<ulonglong2>(), t.n, t.levels, lb, rb, vlb, vrb, nq,
                                                  count_out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_range_report(TreeImpl& t, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                           const uint64_t* vrb, uint64_t nq, const uint64_t* off, uint64_t cap, uint64_t* pos,
                           uint64_t* val, cudaStream_t s) {
  int rc;
  if ((t.flags & WTG_ALL) != WTG_ALL)
    return fail(WTG_ERR_INVALID, "range_search_2d with report needs rank and both selects");
  if (!nq || !cap) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_range_report_kernel<<<qgrid(nq * 32), 256, 0, s>>>(
      t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(), t.node_tab.as<ulonglong2>(), sel_view(t.bv, 1),
      sel_view(t.bv, 0), t.n, t.levels, lb, rb, vlb, vrb, nq, off, cap, pos, val);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_interval_symbols(TreeImpl& t, const uint64_t* i, const uint64_t* j, uint64_t nq, uint64_t* k_out,
                               const uint64_t* off, uint64_t cap, uint64_t* cs, uint64_t* ri, uint64_t* rj,
                               cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "interval_symbols"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  const uint64_t* tree = t.bits.as<uint64_t>();
  const uint64_t* rt = t.bv.rank.as<uint64_t>();
  const ulonglong2* tab = t.node_tab.as<ulonglong2>();
  if (k_out) {
    wt_interval_symbols_kernel<false><<<qgrid(nq), 256, 0, s>>>(tree, rt, tab, t.n, t.levels, i, j, nq, k_out,
                                                                nullptr, 0, nullptr, nullptr, nullptr);
  } else {
    if (!cap) return WTG_OK;
    wt_interval_symbols_kernel<true><<<qgrid(nq), 256, 0, s>>>(tree, rt, tab, t.n, t.levels, i, j, nq, nullptr,
                                                               off, cap, cs, ri, rj);
  }
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_expand(TreeImpl& t, const uint64_t* nodes, uint64_t nn, uint64_t* left, uint64_t* right,
                     cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "expand"))) return rc;
  if (!nn) return WTG_OK;
  wt_expand_kernel<<<qgrid(nn), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(), t.n, t.levels, nodes,
                                             nn, left, right);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_expand_ranges(TreeImpl& t, uint64_t voff, const uint64_t* ranges, uint64_t nr, uint64_t* left,
                            uint64_t* right, cudaStream_t s) {
  int rc;
  if ((rc = need_rank(t, "expand"))) return rc;
  if (!nr) return WTG_OK;
  wt_expand_ranges_kernel<<<qgrid(nr), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                                    (uint64_t)t.levels * t.n, voff, ranges, nr, left, right);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

}  // namespace wtg
