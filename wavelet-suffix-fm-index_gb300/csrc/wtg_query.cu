// wtg_query.cu -- batched queries on the GPU: rank_support_v::rank,
// select_support_mcl::select, and wt_int's access / rank / inverse_select /
// select, one thread per query; plus the alphabet remap helper.
#include <algorithm>

#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {

__device__ __forceinline__ int bit_at(const uint64_t* __restrict__ w, uint64_t p) {
  return (int)((w[p >> 6] >> (p & 63)) & 1);
}

// Node table: for every heap node h of levels 0..L-1 (root 0, children
// 2h+1 / 2h+2), x = global bit offset of the node's start and y = ones before
// it.  These are the `offset` and `o = m_tree_rank(offset)` that wt_int's
// queries recompute at every level (wt_int_par.hpp:527-536, 561-572,
// 596-606); with them tabulated, a query level costs one rank probe and one
// bit word, fetched together with the next level's node entry.
__global__ void node_table_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                  const uint32_t* __restrict__ C, uint64_t n, uint64_t nodes,
                                  ulonglong2* __restrict__ tab) {
  const uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nodes) return;
  const uint64_t l = 63 - __clzll((long long)(h + 1));
  const uint64_t off = l * n + C[h];
  tab[h] = make_ulonglong2(off, rank1_dev(rt, tree, off));
}

// rank1(pos) with the word holding pos already loaded
__device__ __forceinline__ uint64_t rank1_with_word(const uint64_t* __restrict__ rt, uint64_t pos, uint64_t word) {
  const ulonglong2 e = __ldg(reinterpret_cast<const ulonglong2*>(rt) + (pos >> 9));
  uint64_t r = e.x + ((e.y >> (63 - 9 * ((pos & 0x1FF) >> 6))) & 0x1FF);
  if (pos & 63) r += __popcll(word & ((1ull << (pos & 63)) - 1));
  return r;
}

// wt_int::operator[] (wt_int/wt_int_par.hpp:519-541) and inverse_select
// (:588-611): descend by the bit at i; the symbol is the path, the rank the
// final position
template <bool INV>
__global__ void wt_descend_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                                  const ulonglong2* __restrict__ tab, uint64_t n, int L,
                                  const uint64_t* __restrict__ q, uint64_t nq, uint64_t* __restrict__ out,
                                  uint64_t* __restrict__ sym_out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  uint64_t i = q[k];
  if (i >= n) {
    out[k] = NONE64;
    if (INV) sym_out[k] = NONE64;
    return;
  }
  uint64_t h = 0, c = 0;
  ulonglong2 nd = __ldg(tab);
  for (int lv = 0; lv < L; ++lv) {
    const uint64_t pos = nd.x + i;
    ulonglong2 c0 = nd, c1 = nd;
    if (lv + 1 < L) {
      c0 = __ldg(tab + 2 * h + 1);
      c1 = __ldg(tab + 2 * h + 2);
    }
    const uint64_t word = __ldg(tree + (pos >> 6));
    const uint64_t r = rank1_with_word(rt, pos, word) - nd.y;
    const uint64_t bit = (word >> (pos & 63)) & 1;
    c = (c << 1) | bit;
    if (bit) {
      i = r;
      h = 2 * h + 2;
      nd = c1;
    } else {
      i -= r;
      h = 2 * h + 1;
      nd = c0;
    }
  }
  if (INV) {
    out[k] = i;
    sym_out[k] = c;
  } else {
    out[k] = c;
  }
}

// wt_int::rank (wt_int_par.hpp:553-577): descend along c's path
__global__ void wt_rank_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt,
                               const ulonglong2* __restrict__ tab, uint64_t n, int L,
                               const uint64_t* __restrict__ q, const uint64_t* __restrict__ sym, uint64_t nq,
                               uint64_t* __restrict__ out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  uint64_t i = q[k];
  const uint64_t c = sym[k];
  if (i > n) {
    out[k] = NONE64;
    return;
  }
  if (L < 64 && (1ull << L) <= c) {
    out[k] = 0;
    return;
  }
  uint64_t h = 0;
  ulonglong2 nd = __ldg(tab);
  for (int lv = 0; lv < L && i; ++lv) {
    const uint64_t bit = (c >> (L - 1 - lv)) & 1;
    const uint64_t child = 2 * h + 1 + bit;
    ulonglong2 next = nd;
    if (lv + 1 < L) next = __ldg(tab + child);
    const uint64_t pos = nd.x + i;
    const uint64_t word = __ldg(tree + (pos >> 6));
    const uint64_t r = rank1_with_word(rt, pos, word) - nd.y;
    i = bit ? r : i - r;
    h = child;
    nd = next;
  }
  out[k] = i;
}

// wt_int::select (wt_int_par.hpp:622-660)
__global__ void wt_select_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt, SelView s1,
                                 SelView s0, uint64_t n, int L, const uint64_t* __restrict__ q,
                                 const uint64_t* __restrict__ sym, uint64_t nq, uint64_t* __restrict__ out) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  uint64_t i = q[k];
  const uint64_t c = sym[k];
  uint64_t path_off[25], path_rank[25];
  uint64_t offset = 0, mask = 1ull << (L - 1), node_size = n;
  path_off[0] = path_rank[0] = 0;
  if (i == 0 || (L < 64 && (1ull << L) <= c)) {
    out[k] = NONE64;
    return;
  }
  for (int lv = 0; lv < L && node_size; ++lv) {
    const uint64_t o = rank1_dev(rt, tree, offset);
    path_rank[lv] = o;
    const uint64_t oe = rank1_dev(rt, tree, offset + node_size) - o;
    if (c & mask) {
      offset += node_size - oe;
      node_size = oe;
    } else {
      node_size = node_size - oe;
    }
    offset += n;
    path_off[lv + 1] = offset;
    mask >>= 1;
  }
  if (node_size == 0 || node_size < i) {
    out[k] = NONE64;  // the reference throws std::logic_error here
    return;
  }
  mask = 1;
  for (int lv = L; lv > 0; --lv) {
    offset = path_off[lv - 1];
    const uint64_t o = path_rank[lv - 1];
    if (c & mask) i = select_dev(s1, o + i) - offset + 1;
    else i = select_dev(s0, offset - o + i) - offset + 1;
    mask <<= 1;
  }
  out[k] = i - 1;
}

__global__ void bv_rank_kernel(const uint64_t* __restrict__ words, const uint64_t* __restrict__ rt, uint64_t size,
                               const uint64_t* __restrict__ q, uint64_t nq, uint64_t* __restrict__ out) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  const uint64_t idx = q[k];
  out[k] = idx <= size ? rank1_dev(rt, words, idx) : NONE64;
}

__global__ void bv_select_kernel(SelView v, const uint64_t* __restrict__ q, uint64_t nq, uint64_t* __restrict__ out) {
  uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  out[k] = select_dev(v, q[k]);
}

static unsigned qgrid(uint64_t nq) { return (unsigned)((nq + 255) / 256); }

static int need(const TreeImpl& t, uint32_t f, const char* what) {
  if ((t.flags & f) != f) return fail(WTG_ERR_INVALID, std::string(what) + " needs a tree built with the supports it uses");
  return WTG_OK;
}

int tree_node_table(TreeImpl& t, cudaStream_t s) {
  int rc;
  if (t.node_tab_ok) return WTG_OK;
  const uint64_t nodes = (1ull << t.levels) - 1;
  if ((rc = t.node_tab.ensure(nodes * sizeof(ulonglong2), s))) return rc;
  const uint64_t heap = 1ull << t.levels;
  node_table_kernel<<<(unsigned)((nodes + 255) / 256), 256, 0, s>>>(
      t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(), t.zeros.as<uint32_t>() + 2 * heap, t.n, nodes,
      t.node_tab.as<ulonglong2>());
  count_launch();
  WTG_CK(cudaGetLastError());
  t.node_tab_ok = true;
  return WTG_OK;
}

int launch_wt_access(TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s) {
  int rc;
  if ((rc = need(t, WTG_RANK, "access"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_descend_kernel<false><<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                                    t.node_tab.as<ulonglong2>(), t.n, t.levels, idx, nq, out,
                                                    nullptr);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_rank(TreeImpl& t, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out,
                   cudaStream_t s) {
  int rc;
  if ((rc = need(t, WTG_RANK, "rank"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_rank_kernel<<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                           t.node_tab.as<ulonglong2>(), t.n, t.levels, idx, sym, nq, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_inverse_select(TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* rank_out,
                             uint64_t* sym_out, cudaStream_t s) {
  int rc;
  if ((rc = need(t, WTG_RANK, "inverse_select"))) return rc;
  if (!nq) return WTG_OK;
  if ((rc = tree_node_table(t, s))) return rc;
  wt_descend_kernel<true><<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(),
                                                   t.node_tab.as<ulonglong2>(), t.n, t.levels, idx, nq, rank_out,
                                                   sym_out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_wt_select(const TreeImpl& t, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out,
                     cudaStream_t s) {
  if (int rc = need(t, WTG_ALL, "select")) return rc;
  if (!nq) return WTG_OK;
  wt_select_kernel<<<qgrid(nq), 256, 0, s>>>(t.bits.as<uint64_t>(), t.bv.rank.as<uint64_t>(), sel_view(t.bv, 1),
                                            sel_view(t.bv, 0), t.n, t.levels, i, sym, nq, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_bv_rank(const BvSupport& bv, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s) {
  if (!(bv.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "rank needs WTG_RANK");
  if (!nq) return WTG_OK;
  bv_rank_kernel<<<qgrid(nq), 256, 0, s>>>(bv.words, bv.rank.as<uint64_t>(), bv.size, idx, nq, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_bv_select(const BvSupport& bv, int t_b, const uint64_t* i, uint64_t nq, uint64_t* out, cudaStream_t s) {
  if (!(bv.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select needs its support built");
  if (!nq) return WTG_OK;
  bv_select_kernel<<<qgrid(nq), 256, 0, s>>>(sel_view(bv, t_b), i, nq, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

// ---------------------------------------------------------- alphabet remap

template <typename T>
__global__ void remap_mark_kernel(const T* __restrict__ s, uint64_t n, uint32_t* __restrict__ flag) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    flag[(uint64_t)s[i]] = 1;
}

template <typename T>
__global__ void remap_apply_kernel(T* __restrict__ s, uint64_t n, const uint32_t* __restrict__ rank) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    s[i] = (T)rank[(uint64_t)s[i]];
}

template <typename T>
__global__ void remap_max_kernel(const T* __restrict__ s, uint64_t n, unsigned long long* out) {
  uint64_t m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t x = s[i];
    m = x > m ? x : m;
  }
  atomicMax(out, (unsigned long long)m);
}

template <typename T>
static int remap_t(T* d, uint64_t n, uint64_t* sigma, DevBuf& tmp, DevBuf& scan_tmp, uint32_t* d_err,
                   cudaStream_t s) {
  int rc;
  unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 8);
  if (grid == 0) grid = 1;
  if ((rc = tmp.ensure(sizeof(unsigned long long), s))) return rc;
  WTG_CK(cudaMemsetAsync(tmp.p, 0, sizeof(unsigned long long), s));
  remap_max_kernel<T><<<grid, 256, 0, s>>>(d, n, tmp.as<unsigned long long>());
  count_launch();
  WTG_CK(cudaGetLastError());
  unsigned long long mx = 0;
  WTG_CK(cudaMemcpyAsync(&mx, tmp.p, sizeof(mx), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  if (mx >= (1ull << 31)) return fail(WTG_ERR_RANGE, "remap: symbol values must be below 2^31");
  const uint64_t k = mx + 2;  // flags for values 0..max, plus the total
  if ((rc = tmp.ensure(k * sizeof(uint32_t), s))) return rc;
  uint32_t* flag = tmp.as<uint32_t>();
  WTG_CK(cudaMemsetAsync(flag, 0, k * sizeof(uint32_t), s));
  remap_mark_kernel<T><<<grid, 256, 0, s>>>(d, n, flag);
  count_launch();
  WTG_CK(cudaGetLastError());
  if ((rc = scan_exclusive_u32(flag, flag, k, scan_tmp, d_err, s))) return rc;
  remap_apply_kernel<T><<<grid, 256, 0, s>>>(d, n, flag);
  count_launch();
  WTG_CK(cudaGetLastError());
  uint32_t sg = 0;
  WTG_CK(cudaMemcpyAsync(&sg, flag + (k - 1), sizeof(sg), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  *sigma = sg;
  return WTG_OK;
}

int remap_alphabet_device(void* d_seq, uint64_t n, int eb, uint64_t* sigma, DevBuf& tmp, DevBuf& scan_tmp,
                          uint32_t* d_err, cudaStream_t s) {
  if (n == 0) {
    *sigma = 0;
    return WTG_OK;
  }
  switch (eb) {
    case 1: return remap_t<uint8_t>((uint8_t*)d_seq, n, sigma, tmp, scan_tmp, d_err, s);
    case 2: return remap_t<uint16_t>((uint16_t*)d_seq, n, sigma, tmp, scan_tmp, d_err, s);
    case 4: return remap_t<uint32_t>((uint32_t*)d_seq, n, sigma, tmp, scan_tmp, d_err, s);
    default: return remap_t<uint64_t>((uint64_t*)d_seq, n, sigma, tmp, scan_tmp, d_err, s);
  }
}

}  // namespace wtg
