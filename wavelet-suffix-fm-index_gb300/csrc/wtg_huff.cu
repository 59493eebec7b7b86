// wtg_huff.cu -- Huffman-shaped wavelet tree of a byte text on the GPU: the
// tree sdsl::wt_huff<> builds (wt_huff/wt_huff_par.hpp), the one the
// reference's FM-index uses (fm-index/par/WT.C:44).
//
// Shape (wt_huff/wt_huff_par.hpp:82-117): the byte counts go into a
// min-priority queue of (frequency, node number) pairs -- leaves numbered by
// increasing byte value, merged nodes numbered after them; the two smallest
// pairs merge until one node is left.  The tree is laid out breadth first
// (root 0, a node's left child before its right), each inner node's
// bitvector starts where the sizes of the inner nodes before it add up to
// (bv_pos), and a byte's code is its path from the root (bit d: the (d+1)-th
// edge goes right).  The shape has at most 511 nodes and is made on the host
// from the device histogram.
//
// Bits (wt_huff/wt_pc_par.hpp:193-258): node v's bitvector holds, in text
// order, the next code bit of every symbol whose path passes v.  Breadth
// first, the inner nodes of one depth are consecutive, left to right, so the
// bits of depth d are one run [D_d, D_{d+1}) filled from the "depth-d
// sequence": the symbols whose code is longer than d, stably ordered by their
// depth-d node.  One pass per depth:
//   huff_bits_kernel    the run's bits (one ballot per 32 symbols) and the
//                       zero count of every 512-symbol chunk;
//   (scan of the chunk counts)
//   huff_node_kernel    per inner node of the depth, the scatter constants of
//                       its children: the next sequence position of the first
//                       symbol going left / right, minus the zeros / ones
//                       before the node;
//   huff_scatter_kernel every symbol whose child is an inner node goes to
//                       base + (zeros or ones before it at this depth); a
//                       symbol reaching a leaf leaves the sequence.
// rank_support_v and select_support_mcl over the bitvector come from the
// generic bitvector build; the node ranks (bv_pos_rank) from the rank table.
// The queries follow wt_pc (wt_huff/wt_pc_par.hpp:430-552).
#include <algorithm>
#include <queue>
#include <vector>

#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {

constexpr int HUFF_MAX_NODES = 511;
constexpr uint16_t HUFF_NONE = 0xFFFF;
constexpr int HUFF_THREADS = 256;
constexpr int HUFF_CHUNK = 512;  // symbols per warp chunk

struct HuffNodeDev {
  uint64_t bv_pos;
  uint64_t rank;       // ones before bv_pos (inner), the byte (leaf)
  uint16_t parent, child0, child1, leaf;  // leaf: 1 for a leaf
};

struct HuffImpl {
  uint64_t n = 0, sigma = 0, size = 0;
  int maxlen = 0;
  uint32_t flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  struct Node {
    uint64_t bv_pos = 0, freq = 0, sym = 0;
    int parent = -1, child[2] = {-1, -1}, depth = 0;
  };
  std::vector<Node> nodes;
  uint64_t path[256] = {0};
  int len[256] = {0};
  int leaf[256];
  DevBuf text, seq[2], bits, chunkz, chunkpre, scan_tmp, err, hist, dnodes, dpath, dnode_at, nbase, ids, qbuf;
  BvSupport bv;
  HuffImpl() { std::fill(leaf, leaf + 256, -1); }
};

namespace {

__global__ void huff_hist_kernel(const uint8_t* __restrict__ s, uint64_t n, unsigned long long* __restrict__ hist) {
  __shared__ uint32_t h[256];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[s[i]], 1u);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

// the depth-d bits of a warp's 512-symbol chunk: bit of symbol i at global
// position D + i (ORed, as runs need not start on a word); its zero count
__global__ void __launch_bounds__(HUFF_THREADS)
    huff_bits_kernel(const uint8_t* __restrict__ src, uint64_t cnt, int d, const uint64_t* __restrict__ path,
                     uint64_t D, uint64_t* __restrict__ bits, uint32_t* __restrict__ chunkz) {
  __shared__ uint64_t s_path[256];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) s_path[i] = path[i];
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nchunks = (cnt + HUFF_CHUNK - 1) / HUFF_CHUNK;
  const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = w0; c < nchunks; c += nw) {
    uint32_t zeros = 0;
    for (int r = 0; r < HUFF_CHUNK / 32; ++r) {
      const uint64_t i = c * HUFF_CHUNK + 32 * r + lane;
      const bool valid = i < cnt;
      const uint32_t b = valid ? (uint32_t)((s_path[src[i]] >> d) & 1u) : 0u;
      const uint32_t row = __ballot_sync(0xffffffffu, b);
      zeros += __popc(__ballot_sync(0xffffffffu, valid && !b));
      if (lane == 0 && row) {
        const uint64_t p = D + c * HUFF_CHUNK + 32 * r;
        const uint32_t sh = (uint32_t)(p & 63);
        atomicOr((unsigned long long*)&bits[p >> 6], (unsigned long long)row << sh);
        if (sh > 32) atomicOr((unsigned long long*)&bits[(p >> 6) + 1], (unsigned long long)row >> (64 - sh));
      }
    }
    if (lane == 0) chunkz[c] = zeros;
  }
}

// scatter constants of the children of depth-d inner node v: left child gets
// the symbols going 0 at base0 + (zeros before them at this depth), right
// child the 1s at base1 + (ones before them), modulo 2^64 (unused for a leaf
// child)
__global__ void huff_node_kernel(const HuffNodeDev* __restrict__ nodes, const uint16_t* __restrict__ ids, int count,
                                 uint64_t D, uint64_t Dnext, const uint32_t* __restrict__ chunkpre,
                                 const uint64_t* __restrict__ bits, uint64_t* __restrict__ nbase) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint16_t v = ids[k];
  const uint64_t start = nodes[v].bv_pos - D;  // the node's first position in the depth-d sequence
  // zeros before it: the chunk's prefix plus the zeros of the run in [chunk start, start)
  uint64_t z = chunkpre[start / HUFF_CHUNK];
  for (uint64_t p = D + (start & ~(uint64_t)(HUFF_CHUNK - 1)); p < D + start;) {
    const uint64_t w = bits[p >> 6];
    const uint32_t lo = (uint32_t)(p & 63);
    const uint32_t take = (uint32_t)min((uint64_t)(64 - lo), D + start - p);
    const uint64_t m = (take == 64 ? ~0ull : ((1ull << take) - 1)) << lo;
    z += take - __popcll(w & m);
    p += take;
  }
  const uint16_t c0 = nodes[v].child0, c1 = nodes[v].child1;
  nbase[2 * v] = (nodes[c0].bv_pos - Dnext) - z;
  nbase[2 * v + 1] = (nodes[c1].bv_pos - Dnext) - (start - z);
}

__global__ void __launch_bounds__(HUFF_THREADS)
    huff_scatter_kernel(const uint8_t* __restrict__ src, uint64_t cnt, int d, const uint64_t* __restrict__ path,
                        const uint16_t* __restrict__ node_at, const uint32_t* __restrict__ chunkpre,
                        const uint64_t* __restrict__ nbase, uint8_t* __restrict__ dst, uint64_t cnt_next,
                        uint32_t* __restrict__ err) {
  __shared__ uint64_t s_path[256];
  __shared__ uint16_t s_node[256];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
    s_path[i] = path[i];
    s_node[i] = node_at[(uint64_t)d * 256 + i];
  }
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1;
  const uint64_t nchunks = (cnt + HUFF_CHUNK - 1) / HUFF_CHUNK;
  const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t c = w0; c < nchunks; c += nw) {
    uint64_t z = chunkpre[c];  // zeros before the chunk at this depth
    bool bad = false;
    for (int r = 0; r < HUFF_CHUNK / 32; ++r) {
      const uint64_t i = c * HUFF_CHUNK + 32 * r + lane;
      const bool valid = i < cnt;
      const uint8_t x = valid ? src[i] : 0;
      const uint32_t b = valid ? (uint32_t)((s_path[x] >> d) & 1u) : 0u;
      const uint32_t zm = __ballot_sync(0xffffffffu, valid && !b);
      const uint64_t zb = z + __popc(zm & lt);  // zeros before symbol i
      z += __popc(zm);
      // a symbol whose code ends at depth d + 1 reaches a leaf and leaves the
      // sequence (bases are modular: no base value can mark a leaf child)
      if (valid && (uint32_t)(s_path[x] >> 56) > (uint32_t)d + 1) {
        const uint64_t dest = nbase[2 * s_node[x] + b] + (b ? i - zb : zb);
        if (dest < cnt_next) dst[dest] = x;
        else bad = true;
      }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicCAS(err, 0u, (uint32_t)DERR_BAD_INDEX);
  }
}

__global__ void huff_node_rank_kernel(HuffNodeDev* __restrict__ nodes, int count, const uint64_t* __restrict__ rt,
                                      const uint64_t* __restrict__ bits) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= count || nodes[v].leaf) return;
  nodes[v].rank = rank1_dev(rt, bits, nodes[v].bv_pos);
}

struct HuffView {
  const HuffNodeDev* nodes;
  const uint64_t* path;  // per byte: code | length << 56
  const uint16_t* leaf;  // per byte: leaf node or HUFF_NONE
  const uint64_t* bits;
  const uint64_t* rt;
  SelView s1, s0;
  uint64_t n, sigma;
};

__device__ __forceinline__ uint32_t huff_bit(const uint64_t* bits, uint64_t p) { return (bits[p >> 6] >> (p & 63)) & 1u; }

// operator[] (wt_huff/wt_pc_par.hpp:430-448); with INV, inverse_select
// (:498-514): the rank of the symbol at i among its occurrences before i
template <bool INV>
__global__ void huff_access_kernel(HuffView v, const uint64_t* __restrict__ q, uint64_t nq, uint64_t* __restrict__ out,
                                   uint64_t* __restrict__ sym_out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  uint64_t i = q[k];
  if (i >= v.n) {
    out[k] = NONE64;
    if (INV) sym_out[k] = NONE64;
    return;
  }
  uint16_t u = 0;
  while (!v.nodes[u].leaf) {
    const uint64_t p = v.nodes[u].bv_pos + i;
    const uint64_t r = rank1_dev(v.rt, v.bits, p) - v.nodes[u].rank;
    if (huff_bit(v.bits, p)) {
      i = r;
      u = v.nodes[u].child1;
    } else {
      i -= r;
      u = v.nodes[u].child0;
    }
  }
  if (INV) {
    out[k] = i;
    sym_out[k] = v.nodes[u].rank;
  } else {
    out[k] = v.nodes[u].rank;
  }
}

// rank(i, c) (wt_huff/wt_pc_par.hpp:463-484): occurrences of c in [0, i)
__device__ __forceinline__ uint64_t huff_rank_dev(const HuffView& v, uint64_t i, uint32_t c) {
  if (c > 255 || v.leaf[c] == HUFF_NONE) return 0;
  if (v.sigma == 1) return i;
  uint64_t p = v.path[c];
  const uint32_t len = (uint32_t)(p >> 56);
  uint64_t res = i;
  uint16_t u = 0;
  for (uint32_t l = 0; l < len && res; ++l, p >>= 1) {
    const uint64_t r = rank1_dev(v.rt, v.bits, v.nodes[u].bv_pos + res) - v.nodes[u].rank;
    res = (p & 1) ? r : res - r;
    u = (p & 1) ? v.nodes[u].child1 : v.nodes[u].child0;
  }
  return res;
}

__global__ void huff_rank_kernel(HuffView v, const uint64_t* __restrict__ qi, const uint64_t* __restrict__ qc,
                                 uint64_t nq, uint64_t* __restrict__ out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  const uint64_t i = qi[k];
  out[k] = i > v.n ? NONE64 : huff_rank_dev(v, i, qc[k] > 255 ? 256u : (uint32_t)qc[k]);
}

// select(i, c) (wt_huff/wt_pc_par.hpp:527-552): from c's leaf up, select1 /
// select0 on the bitvector; n where c does not occur; UINT64_MAX where c
// occurs fewer than i times (the reference asserts)
__global__ void huff_select_kernel(HuffView v, const uint64_t* __restrict__ qi, const uint64_t* __restrict__ qc,
                                   uint64_t nq, uint64_t* __restrict__ out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nq) return;
  const uint64_t i = qi[k], c = qc[k];
  if (c > 255 || v.leaf[c] == HUFF_NONE) {
    out[k] = v.n;
    return;
  }
  if (i == 0 || i > huff_rank_dev(v, v.n, (uint32_t)c)) {
    out[k] = NONE64;
    return;
  }
  if (v.sigma == 1) {
    out[k] = i - 1;
    return;
  }
  uint16_t u = v.leaf[c];
  uint64_t res = i - 1;
  while (u != 0) {
    const uint16_t par = v.nodes[u].parent;
    const uint64_t bp = v.nodes[par].bv_pos, br = v.nodes[par].rank;
    uint64_t s;
    if (v.nodes[par].child1 == u) s = select_dev(v.s1, br + res + 1);
    else s = select_dev(v.s0, bp - br + res + 1);
    if (s == NONE64) {
      res = NONE64;
      break;
    }
    res = s - bp;
    u = par;
  }
  out[k] = res;
}

// backward search over the BWT's Huffman-shaped tree: per pattern (bytes
// pat[off[q] .. off[q + 1])) the rows [sp, ep) prefixed by it, C[c] = bytes
// below c in the text
__global__ void huff_fm_count_kernel(HuffView v, const uint64_t* __restrict__ C, const uint8_t* __restrict__ pat,
                                     const uint64_t* __restrict__ off, uint64_t npat, uint64_t* __restrict__ out) {
  const uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npat) return;
  uint64_t sp = 0, ep = v.n;
  for (uint64_t j = off[q + 1]; j > off[q] && sp < ep;) {
    --j;
    const uint32_t c = pat[j];
    if (v.leaf[c] == HUFF_NONE) {
      sp = ep = 0;
      break;
    }
    sp = C[c] + huff_rank_dev(v, sp, c);
    ep = C[c] + huff_rank_dev(v, ep, c);
  }
  out[q] = ep > sp ? ep - sp : 0;
}

unsigned hgrid(uint64_t items, unsigned per, unsigned cap) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + per - 1) / per, cap));
}

}  // namespace

HuffImpl* huff_new() { return new (std::nothrow) HuffImpl(); }

void huff_delete(HuffImpl* h) {
  if (!h) return;
  cudaStream_t s = h->stream;
  DevBuf* bufs[] = {&h->text, &h->seq[0], &h->seq[1], &h->bits, &h->chunkz, &h->chunkpre, &h->scan_tmp, &h->err,
                    &h->hist, &h->dnodes, &h->dpath, &h->dnode_at, &h->nbase, &h->ids, &h->qbuf};
  for (DevBuf* d : bufs) d->release(s);
  bv_release(h->bv, s);
  cudaStreamSynchronize(s);
  if (h->own_stream) cudaStreamDestroy(s);
  delete h;
}

cudaStream_t huff_stream(const HuffImpl& h) { return h.stream; }

// the shape and breadth-first layout of the code tree from the byte counts
static void huff_shape(HuffImpl& h, const uint64_t* counts) {
  struct S {
    uint64_t freq, sym;
    int c0, c1;
  };
  std::vector<S> shape;
  typedef std::pair<uint64_t, uint64_t> FI;  // (frequency, node number)
  std::priority_queue<FI, std::vector<FI>, std::greater<FI>> pq;
  for (uint32_t c = 0; c < 256; ++c)
    if (counts[c]) {
      pq.push(FI(counts[c], shape.size()));
      shape.push_back({counts[c], c, -1, -1});
    }
  while (pq.size() > 1) {
    const FI a = pq.top();
    pq.pop();
    const FI b = pq.top();
    pq.pop();
    pq.push(FI(a.first + b.first, shape.size()));
    shape.push_back({a.first + b.first, 0, (int)a.second, (int)b.second});
  }
  h.nodes.clear();
  h.sigma = 0;
  std::fill(h.leaf, h.leaf + 256, -1);
  std::fill(h.path, h.path + 256, 0ull);
  std::fill(h.len, h.len + 256, 0);
  h.size = 0;
  h.maxlen = 0;
  if (shape.empty()) return;
  std::vector<int> from(1, (int)shape.size() - 1);  // breadth-first index -> shape index
  h.nodes.resize(1);
  for (size_t k = 0; k < from.size(); ++k) {  // the placed nodes are the queue
    const S& sn = shape[from[k]];
    h.nodes[k].bv_pos = h.size;
    h.nodes[k].freq = sn.freq;
    h.nodes[k].sym = sn.sym;
    if (sn.c0 >= 0) {
      h.size += sn.freq;
      for (int j = 0; j < 2; ++j) {
        const int id = (int)from.size();
        from.push_back(j ? sn.c1 : sn.c0);
        HuffImpl::Node child;
        child.parent = (int)k;
        child.depth = h.nodes[k].depth + 1;
        h.nodes.push_back(child);
        h.nodes[k].child[j] = id;
      }
    } else {
      h.leaf[sn.sym] = (int)k;
      ++h.sigma;
    }
  }
  for (uint32_t c = 0; c < 256; ++c) {
    if (h.leaf[c] < 0) continue;
    uint64_t p = 0;
    int len = 0;
    for (int u = h.leaf[c]; u != 0; u = h.nodes[u].parent) {
      p = (p << 1) | (h.nodes[h.nodes[u].parent].child[1] == u ? 1u : 0u);
      ++len;
    }
    h.path[c] = p;
    h.len[c] = len;
    h.maxlen = std::max(h.maxlen, len);
  }
}

int huff_build(HuffImpl& h, const uint8_t* d_text, uint64_t n, uint32_t flags) {
  int rc;
  cudaStream_t s = h.stream;
  if (n >= (1ull << 40)) return fail(WTG_ERR_INVALID, "text too large");
  if (flags & ~WTG_ALL) return fail(WTG_ERR_INVALID, "unknown flags");
  if (flags & (WTG_SELECT1 | WTG_SELECT0)) flags |= WTG_RANK;  // the node ranks and selects read the rank table
  h.n = n;
  h.flags = flags;
  if ((rc = h.err.ensure(sizeof(uint32_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(h.err.p, 0, sizeof(uint32_t), s));
  uint32_t* d_err = h.err.as<uint32_t>();
  // histogram -> shape (host)
  if ((rc = h.hist.ensure(256 * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(h.hist.p, 0, 256 * sizeof(uint64_t), s));
  if (n) {
    huff_hist_kernel<<<hgrid(n, 256 * 16, 152 * 8), 256, 0, s>>>(d_text, n, h.hist.as<unsigned long long>());
    count_launch();
    WTG_CK(cudaGetLastError());
  }
  uint64_t counts[256];
  WTG_CK(cudaMemcpyAsync(counts, h.hist.p, sizeof(counts), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  huff_shape(h, counts);
  const int nn = (int)h.nodes.size();
  if (nn > HUFF_MAX_NODES) return fail(WTG_ERR_INVALID, "a byte alphabet's Huffman shape has at most 511 nodes");
  const uint64_t W = (h.size + 63) / 64;
  if ((rc = h.bits.ensure((W + 2) * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemsetAsync(h.bits.p, 0, (W + 2) * sizeof(uint64_t), s));
  // node table, codes, and per depth the node on each byte's path
  std::vector<HuffNodeDev> hn(std::max(nn, 1));
  for (int v = 0; v < nn; ++v) {
    const HuffImpl::Node& u = h.nodes[v];
    hn[v].bv_pos = u.bv_pos;
    hn[v].rank = u.child[0] < 0 ? u.sym : 0;
    hn[v].parent = u.parent < 0 ? HUFF_NONE : (uint16_t)u.parent;
    hn[v].child0 = u.child[0] < 0 ? HUFF_NONE : (uint16_t)u.child[0];
    hn[v].child1 = u.child[1] < 0 ? HUFF_NONE : (uint16_t)u.child[1];
    hn[v].leaf = u.child[0] < 0 ? 1 : 0;
  }
  uint64_t pl[256];
  uint16_t lf[256];
  for (int c = 0; c < 256; ++c) {
    pl[c] = h.path[c] | ((uint64_t)h.len[c] << 56);
    lf[c] = h.leaf[c] < 0 ? HUFF_NONE : (uint16_t)h.leaf[c];
  }
  const int depths = std::max(h.maxlen, 1);
  std::vector<uint16_t> node_at((size_t)depths * 256, HUFF_NONE);
  for (int c = 0; c < 256; ++c) {
    if (h.leaf[c] < 0) continue;
    int u = 0;
    for (int d = 0; d < h.len[c]; ++d) {
      node_at[(size_t)d * 256 + c] = (uint16_t)u;
      u = h.nodes[u].child[(h.path[c] >> d) & 1];
    }
  }
  if ((rc = h.dnodes.ensure(hn.size() * sizeof(HuffNodeDev), s))) return rc;
  if ((rc = h.dpath.ensure(256 * (sizeof(uint64_t) + sizeof(uint16_t)), s))) return rc;
  if ((rc = h.dnode_at.ensure(node_at.size() * sizeof(uint16_t), s))) return rc;
  if ((rc = h.nbase.ensure(2 * std::max(nn, 1) * sizeof(uint64_t), s))) return rc;
  WTG_CK(cudaMemcpyAsync(h.dnodes.p, hn.data(), hn.size() * sizeof(HuffNodeDev), cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(h.dpath.p, pl, sizeof(pl), cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync((uint8_t*)h.dpath.p + sizeof(pl), lf, sizeof(lf), cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(h.dnode_at.p, node_at.data(), node_at.size() * sizeof(uint16_t), cudaMemcpyHostToDevice,
                         s));
  // per depth: its inner nodes (breadth-first order), the run start D and the sequence length
  std::vector<std::vector<uint16_t>> inner(depths + 1);
  for (int v = 0; v < nn; ++v)
    if (h.nodes[v].child[0] >= 0) inner[h.nodes[v].depth].push_back((uint16_t)v);
  std::vector<uint64_t> D(depths + 2, h.size), cntd(depths + 2, 0);
  for (int d = 0; d <= depths; ++d)
    if (!inner[d].empty()) {
      D[d] = h.nodes[inner[d][0]].bv_pos;
      for (uint16_t v : inner[d]) cntd[d] += h.nodes[v].freq;
    }
  std::vector<uint16_t> ids;
  for (int d = 0; d <= depths; ++d) ids.insert(ids.end(), inner[d].begin(), inner[d].end());
  DevBuf& dids = h.ids;
  if ((rc = dids.ensure(std::max<size_t>(ids.size(), 1) * sizeof(uint16_t), s))) return rc;
  if (!ids.empty())
    WTG_CK(cudaMemcpyAsync(dids.p, ids.data(), ids.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, s));
  if (n && h.size) {
    if ((rc = h.seq[0].ensure(n, s))) return rc;
    if ((rc = h.seq[1].ensure(n, s))) return rc;
    const uint64_t nch = (n + HUFF_CHUNK - 1) / HUFF_CHUNK;
    if ((rc = h.chunkz.ensure((nch + 1) * sizeof(uint32_t), s))) return rc;
    if ((rc = h.chunkpre.ensure((nch + 1) * sizeof(uint32_t), s))) return rc;
    const uint8_t* src = d_text;
    size_t idoff = 0;
    for (int d = 0; d < depths && cntd[d]; ++d) {
      const uint64_t cnt = cntd[d], chunks = (cnt + HUFF_CHUNK - 1) / HUFF_CHUNK;
      const unsigned grid = hgrid(chunks, HUFF_THREADS / 32, 152 * 16);
      huff_bits_kernel<<<grid, HUFF_THREADS, 0, s>>>(src, cnt, d, h.dpath.as<uint64_t>(), D[d],
                                                     h.bits.as<uint64_t>(), h.chunkz.as<uint32_t>());
      count_launch();
      WTG_CK(cudaGetLastError());
      if ((rc = scan_exclusive_u32(h.chunkz.as<uint32_t>(), h.chunkpre.as<uint32_t>(), chunks, h.scan_tmp, d_err,
                                   s)))
        return rc;
      const int cnt_nodes = (int)inner[d].size();
      if (d + 1 < depths && cntd[d + 1]) {
        huff_node_kernel<<<(cnt_nodes + 127) / 128, 128, 0, s>>>(
            h.dnodes.as<HuffNodeDev>(), dids.as<uint16_t>() + idoff, cnt_nodes, D[d], D[d + 1],
            h.chunkpre.as<uint32_t>(), h.bits.as<uint64_t>(), h.nbase.as<uint64_t>());
        count_launch();
        WTG_CK(cudaGetLastError());
        uint8_t* dst = h.seq[d & 1].as<uint8_t>();
        huff_scatter_kernel<<<grid, HUFF_THREADS, 0, s>>>(src, cnt, d, h.dpath.as<uint64_t>(),
                                                          h.dnode_at.as<uint16_t>(), h.chunkpre.as<uint32_t>(),
                                                          h.nbase.as<uint64_t>(), dst, cntd[d + 1], d_err);
        count_launch();
        WTG_CK(cudaGetLastError());
        src = dst;
      }
      idoff += cnt_nodes;
    }
  }
  // rank / select supports and the node ranks
  if (flags) {
    if ((rc = bv_build(h.bv, h.bits.as<uint64_t>(), h.size, flags, d_err, s))) return rc;
    if (nn) {
      huff_node_rank_kernel<<<(nn + 127) / 128, 128, 0, s>>>(h.dnodes.as<HuffNodeDev>(), nn,
                                                             h.bv.rank.as<uint64_t>(), h.bits.as<uint64_t>());
      count_launch();
      WTG_CK(cudaGetLastError());
    }
  }
  return WTG_OK;
}

static HuffView huff_view(HuffImpl& h) {
  HuffView v;
  v.nodes = h.dnodes.as<HuffNodeDev>();
  v.path = h.dpath.as<uint64_t>();
  v.leaf = reinterpret_cast<const uint16_t*>(h.dpath.as<uint8_t>() + 256 * sizeof(uint64_t));
  v.bits = h.bits.as<uint64_t>();
  v.rt = h.bv.rank.as<uint64_t>();
  v.s1 = sel_view(h.bv, 1);
  v.s0 = sel_view(h.bv, 0);
  v.n = h.n;
  v.sigma = h.sigma;
  return v;
}

int huff_info(const HuffImpl& h, uint64_t info[5]) {
  info[0] = h.n;
  info[1] = h.sigma;
  info[2] = h.size;
  info[3] = h.nodes.size();
  const uint64_t cap = (h.size + 63) / 64 * 64;
  info[4] = !(h.flags & WTG_RANK) ? 0 : (h.size == 0 ? 2 : ((cap >> 9) + 1) << 1);  // rank table words
  return WTG_OK;
}

BvSupport& huff_bv(HuffImpl& h) { return h.bv; }
const uint64_t* huff_bits(const HuffImpl& h) { return h.bits.as<uint64_t>(); }
DevBuf& huff_text(HuffImpl& h) { return h.text; }
DevBuf& huff_qbuf(HuffImpl& h) { return h.qbuf; }
const uint32_t* huff_err(const HuffImpl& h) { return h.err.as<uint32_t>(); }
void huff_set_stream(HuffImpl& h, cudaStream_t s, bool own) {
  h.stream = s;
  h.own_stream = own;
}

int huff_tree(HuffImpl& h, uint64_t* nodes, uint64_t* leaves, uint64_t* paths) {
  const int nn = (int)h.nodes.size();
  std::vector<HuffNodeDev> hn(std::max(nn, 1));
  if (nn) {
    WTG_CK(cudaMemcpyAsync(hn.data(), h.dnodes.p, nn * sizeof(HuffNodeDev), cudaMemcpyDeviceToHost, h.stream));
    WTG_CK(cudaStreamSynchronize(h.stream));
  }
  for (int v = 0; v < nn; ++v) {
    nodes[5 * v + 0] = hn[v].bv_pos;
    nodes[5 * v + 1] = hn[v].rank;
    nodes[5 * v + 2] = hn[v].parent;
    nodes[5 * v + 3] = hn[v].child0;
    nodes[5 * v + 4] = hn[v].child1;
  }
  for (int c = 0; c < 256; ++c) {
    leaves[c] = h.leaf[c] < 0 ? HUFF_NONE : (uint64_t)h.leaf[c];
    paths[c] = h.path[c] | ((uint64_t)h.len[c] << 56);
  }
  return WTG_OK;
}

int launch_huff_query(HuffImpl& h, int what, const uint64_t* a, const uint64_t* b, uint64_t nq, uint64_t* out,
                      uint64_t* out2, cudaStream_t s) {
  if (!nq) return WTG_OK;
  if (!(h.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "queries need the rank support");
  if (what == 2 && (h.flags & WTG_ALL) != WTG_ALL) return fail(WTG_ERR_INVALID, "select needs WTG_ALL");
  const HuffView v = huff_view(h);
  const unsigned grid = (unsigned)((nq + 255) / 256);
  if (what == 0) huff_access_kernel<false><<<grid, 256, 0, s>>>(v, a, nq, out, nullptr);
  else if (what == 3) huff_access_kernel<true><<<grid, 256, 0, s>>>(v, a, nq, out, out2);
  else if (what == 1) huff_rank_kernel<<<grid, 256, 0, s>>>(v, a, b, nq, out);
  else huff_select_kernel<<<grid, 256, 0, s>>>(v, a, b, nq, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

int launch_huff_fm_count(HuffImpl& h, const uint64_t* C, const uint8_t* pat, const uint64_t* off, uint64_t npat,
                         uint64_t* out, cudaStream_t s) {
  if (!npat) return WTG_OK;
  if (!(h.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "counting needs the rank support");
  huff_fm_count_kernel<<<(unsigned)((npat + 255) / 256), 256, 0, s>>>(huff_view(h), C, pat, off, npat, out);
  count_launch();
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

}  // namespace wtg
