// wtg_tree.cuh -- device-side state of one wavelet tree (internal).
#pragma once
#include "wtg_internal.cuh"

namespace wtg {

// Device memory layout of one tree (all stream-ordered, reused across rebuilds):
//   seq        the input copied from the host (host-input builds only)
//   lvl[0..1]  ping-pong buffers of the level orders, n symbols each
//   bits       ceil(n*L/64) words of level bits + 2 zero words
//   hist       S: exclusive scan of the 2^L key histogram (2^L + 1 x u32)
//   zeros      [Z | ZS]: zeros per heap node and its exclusive scan (2 x 2^L x u32)
//   base       per heap node (C - Zb, zeros + Zb) (2^L x uint2)
//   status     per level: tile counter + look-back status words
//   bv         rank/select supports over `bits`
struct TreeImpl {
  uint64_t n = 0;
  int levels = 0;
  int elem_bytes = 0;
  uint32_t flags = 0;
  uint64_t bit_words = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf seq, lvl[2], bits, hist, zeros, base, status, scan_tmp, err, scratch, nodes, qbuf;
  BvSupport bv;
};

int tree_levels_from_max(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int* levels);
int tree_build(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int L, uint32_t flags);
int tree_nodes(TreeImpl& t, int ib, uint64_t n_entries, void* d_out);
void tree_release(TreeImpl& t);

// query launchers (wtg_query.cu); all arrays are device arrays
int launch_wt_access(const TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s);
int launch_wt_rank(const TreeImpl& t, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out,
                   cudaStream_t s);
int launch_wt_inverse_select(const TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* rank_out,
                             uint64_t* sym_out, cudaStream_t s);
int launch_wt_select(const TreeImpl& t, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out,
                     cudaStream_t s);
int launch_bv_rank(const BvSupport& bv, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s);
int launch_bv_select(const BvSupport& bv, int t_b, const uint64_t* i, uint64_t nq, uint64_t* out,
                     cudaStream_t s);

// alphabet remap (levelWT/WTTime.C:80-94) on a device sequence, in place
int remap_alphabet_device(void* d_seq, uint64_t n, int eb, uint64_t* sigma, DevBuf& tmp, DevBuf& scan_tmp,
                          uint32_t* d_err, cudaStream_t s);

}  // namespace wtg
