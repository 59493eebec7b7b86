// wtg_tree.cuh -- device-side state of one wavelet tree (internal).
#pragma once
#include <vector>

#include "wtg_internal.cuh"

namespace wtg {

struct LselImpl;

// Device memory layout of one tree (all stream-ordered, reused across rebuilds):
//   seq        the input copied from the host (host-input builds only)
//   lvl[0..1]  ping-pong buffers of the level orders, n symbols each
//   bits       ceil(n*L/64) words of level bits + 2 zero words
//   hist       S: exclusive scan of the 2^L key histogram (2^L + 1 x u32)
//   zeros      [Z | ZS]: zeros per heap node and its exclusive scan (2 x 2^L x u32)
//   base       per heap node (C - Zb, zeros + Zb) (2^L x uint2)
//   status     per level: tile counter + look-back status words
//   bv         rank/select supports over `bits`
//   lvl_args   ones before each level start, L + 1 words (filled on first use
//              after a build by tree_level_args)
struct TreeImpl {
  uint64_t n = 0;
  int levels = 0;
  int elem_bytes = 0;
  uint32_t flags = 0;
  uint64_t bit_words = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf seq, lvl[2], bits, hist, zeros, base, status, scan_tmp, err, scratch, nodes, qbuf, qout;
  DevBuf nodecnt;  // per chunk: the node counts of a level pass, then their scans
  BvSupport bv;
  DevBuf lvl_args;
  bool lvl_args_ok = false;
  DevBuf fm_paths;  // per-symbol node paths for FM-index counting
  DevBuf node_tab;  // per heap node: bit offset of its start, ones before it
  bool node_tab_ok = false;
  uint64_t gen = 0;  // builds so far (indexes built on the tree record it)
  // host destinations filled while the build runs (wtg_tree_build_out): the
  // bits of each level are copied on copy_stream as soon as its pass is done
  uint64_t* host_bits = nullptr;
  uint64_t* host_rank = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev = nullptr, rank_ev = nullptr;
  // input arriving in pieces (wtg_tree_build_out from page-locked memory):
  // piece i holds chunks [i * in_piece_chunks, (i + 1) * in_piece_chunks) of
  // 512 symbols and is on the device once in_ev[i] has fired; the pre-pass
  // counts each piece as it lands.  in_pieces = 0: the input is resident.
  static constexpr int IN_PIECES_MAX = 8;
  cudaStream_t in_stream = nullptr;
  cudaEvent_t in_ev[IN_PIECES_MAX] = {};
  int in_pieces = 0;
  uint64_t in_piece_chunks = 0;
  std::vector<LselImpl*> deps;  // learned select indexes reading this tree
};

int tree_levels_from_max(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int* levels);
// page-locked or registered host memory (copies need no staging)
bool host_page_locked(const void* p);
int tree_build(TreeImpl& t, const void* d_seq, uint64_t n, int eb, int L, uint32_t flags);
int tree_nodes(TreeImpl& t, int ib, uint64_t n_entries, void* d_out);
void tree_release(TreeImpl& t);

// query launchers (wtg_query.cu); all arrays are device arrays.  The node
// table the access / rank / inverse_select kernels read is filled on first
// use after a build (tree_node_table).
int tree_node_table(TreeImpl& t, cudaStream_t s);
int launch_wt_access(TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s);
int launch_wt_rank(TreeImpl& t, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out,
                   cudaStream_t s);
int launch_wt_inverse_select(TreeImpl& t, const uint64_t* idx, uint64_t nq, uint64_t* rank_out,
                             uint64_t* sym_out, cudaStream_t s);
int launch_wt_select(const TreeImpl& t, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out,
                     cudaStream_t s);
int launch_bv_rank(const BvSupport& bv, const uint64_t* idx, uint64_t nq, uint64_t* out, cudaStream_t s);
int launch_bv_select(const BvSupport& bv, int t_b, const uint64_t* i, uint64_t nq, uint64_t* out,
                     cudaStream_t s);

// wt_int's range queries (wtg_range.cu); all arrays are device arrays.
// Count-type queries give UINT64_MAX for an invalid query (bounds outside
// the sequence).  Variable-size answers are placed by answer_offsets: the
// exclusive scan (nq + 1 entries, the last the total) of the per-query
// counts, invalid ones read as 0; the fill launches then write query q's
// answers to [off[q], off[q+1]) below cap.
int answer_offsets(const uint64_t* counts, uint64_t nq, uint64_t* off, DevBuf& scratch, uint32_t* d_err,
                   cudaStream_t s);
int launch_wt_lex_count(TreeImpl& t, const uint64_t* i, const uint64_t* j, const uint64_t* c, uint64_t nq,
                        uint64_t* rank_out, uint64_t* smaller_out, uint64_t* greater_out, cudaStream_t s);
int launch_wt_lex_smaller_count(TreeImpl& t, const uint64_t* i, const uint64_t* c, uint64_t nq, uint64_t* rank_out,
                                uint64_t* smaller_out, cudaStream_t s);
int launch_wt_range_count(TreeImpl& t, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                          const uint64_t* vrb, uint64_t nq, uint64_t* count_out, cudaStream_t s);
int launch_wt_range_report(TreeImpl& t, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                           const uint64_t* vrb, uint64_t nq, const uint64_t* off, uint64_t cap, uint64_t* pos,
                           uint64_t* val, cudaStream_t s);
// with k_out: the counts; without: the fill into off / cap / cs / ri / rj
int launch_wt_interval_symbols(TreeImpl& t, const uint64_t* i, const uint64_t* j, uint64_t nq, uint64_t* k_out,
                               const uint64_t* off, uint64_t cap, uint64_t* cs, uint64_t* ri, uint64_t* rj,
                               cudaStream_t s);
int launch_wt_expand(TreeImpl& t, const uint64_t* nodes, uint64_t nn, uint64_t* left, uint64_t* right,
                     cudaStream_t s);
int launch_wt_expand_ranges(TreeImpl& t, uint64_t voff, const uint64_t* ranges, uint64_t nr, uint64_t* left,
                            uint64_t* right, cudaStream_t s);

// per-level select on the tree's concatenated bitvector -- wt_int's select
// step (m_tree_select1/0(args before the node + i) - node offset,
// wt_int_par.hpp:651-656) with the whole level as the node: for each query
// (level, k) the position, inside the level, of the level's k-th one
// (t_b = 1) or zero (t_b = 0); UINT64_MAX when the level has fewer than k
int tree_level_args(TreeImpl& t, cudaStream_t s);
int launch_level_select(TreeImpl& t, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                        uint64_t* out, cudaStream_t s);

// learned select index over the level bitvectors (wtg_lsel.cu).  An index
// registers with its tree; freeing the tree detaches its indexes (their
// queries then fail) and freeing an index unregisters it.
LselImpl* lsel_new();
void lsel_detach_all(TreeImpl& t);
TreeImpl* lsel_tree(const LselImpl& m);  // NULL once the tree was freed
void lsel_delete(LselImpl* m);
int lsel_build(LselImpl& m, TreeImpl& t, uint32_t segments, uint32_t samples, uint32_t max_window,
               cudaStream_t s);
int lsel_info(const LselImpl& m, uint64_t info[8], cudaStream_t s);
int lsel_get_level(const LselImpl& m, int t_b, int level, uint64_t lvl_info[4], uint32_t* rec, uint64_t nseg,
                   cudaStream_t s);
int launch_lsel_query(LselImpl& m, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                      uint64_t* out, cudaStream_t s);

// FM-index counting by backward search over a tree built on a BWT
// (wtg_fm.cu); C, pat, off and out are device arrays
int launch_fm_count(TreeImpl& t, const uint64_t* C, uint64_t sigma, const uint8_t* pat, const uint64_t* off,
                    uint64_t npat, uint64_t* out, cudaStream_t s);

// batched builds of many short texts (wtg_batch.cu)
struct BatchImpl;
BatchImpl* batch_new();
void batch_delete(BatchImpl* b);
int batch_plan(BatchImpl& b, const uint64_t* lengths, uint64_t T, int L, uint32_t flags, cudaStream_t s,
               bool own_stream);
int batch_run(BatchImpl& b);
int batch_set_shape(BatchImpl& b, int tile, int64_t whole_max, int symbols_per_thread);
int batch_sync(BatchImpl& b, uint32_t* err_out);
int batch_text_info(const BatchImpl& b, uint64_t t, uint64_t info[8]);
int batch_select_info(const BatchImpl& b, uint64_t t, int t_b, uint64_t info[8]);
// what: 0 bits, 1 rank, 2 m_superblock words, 3 descriptors, 4 pool
int batch_get(const BatchImpl& b, uint64_t t, int what, int t_b, void* dst, uint64_t nwords);
void* batch_input(BatchImpl& b);
cudaStream_t batch_stream(const BatchImpl& b);
uint64_t batch_total_symbols(const BatchImpl& b);
int batch_shape(const BatchImpl& b, int* tile, int64_t* whole_max, int* symbols_per_thread, uint64_t* whole_texts,
                float* ms, int nms);

// Huffman-shaped wavelet tree of a byte text (wtg_huff.cu)
struct HuffImpl;
HuffImpl* huff_new();
void huff_delete(HuffImpl* h);
void huff_set_stream(HuffImpl& h, cudaStream_t s, bool own);
cudaStream_t huff_stream(const HuffImpl& h);
int huff_build(HuffImpl& h, const uint8_t* d_text, uint64_t n, uint32_t flags);
int huff_info(const HuffImpl& h, uint64_t info[5]);  // n, sigma, bits, nodes, rank words
int huff_tree(HuffImpl& h, uint64_t* nodes, uint64_t* leaves, uint64_t* paths);
BvSupport& huff_bv(HuffImpl& h);
const uint64_t* huff_bits(const HuffImpl& h);
DevBuf& huff_text(HuffImpl& h);
DevBuf& huff_qbuf(HuffImpl& h);
const uint32_t* huff_err(const HuffImpl& h);
// what: 0 access, 1 rank(a, b), 2 select(a, b), 3 inverse_select (out, out2)
int launch_huff_query(HuffImpl& h, int what, const uint64_t* a, const uint64_t* b, uint64_t nq, uint64_t* out,
                      uint64_t* out2, cudaStream_t s);
int launch_huff_fm_count(HuffImpl& h, const uint64_t* C, const uint8_t* pat, const uint64_t* off, uint64_t npat,
                         uint64_t* out, cudaStream_t s);

// sdsl serialize() streams (wtg_serialize.cu): with dst NULL only *len is
// set; otherwise dst (host memory, cap bytes) receives the stream
int tree_leaf_count(TreeImpl& t, uint64_t* sigma, cudaStream_t s);
int tree_serialize(TreeImpl& t, uint8_t* dst, uint64_t cap, uint64_t* len);
int bv_serialize(BvSupport& bv, uint32_t part, uint8_t* dst, uint64_t cap, uint64_t* len, cudaStream_t s);

// alphabet remap (levelWT/WTTime.C:80-94) on a device sequence, in place
int remap_alphabet_device(void* d_seq, uint64_t n, int eb, uint64_t* sigma, DevBuf& tmp, DevBuf& scan_tmp,
                          uint32_t* d_err, cudaStream_t s);

}  // namespace wtg
