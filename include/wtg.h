/*
 * wtg.h -- C ABI of the GB300 wavelet-tree / rank / select library (libwtg.so).
 *
 * Drop-in boundary for the wavelet-tree construction path of
 * jlabeit/wavelet-suffix-fm-index.  Every entry point is extern "C", takes
 * plain pointers and sizes, never throws, and returns an int status
 * (WTG_OK = 0).  wtg_last_error() gives the message of the calling thread's
 * last failure.  All compute runs as hand-written CUDA kernels on the current
 * CUDA device; there is no CPU fallback: without a usable GPU every build
 * fails with WTG_ERR_CUDA.
 *
 * Layouts (bit-exact with the reference):
 *   bits   : level l of the tree occupies bits [l*n, (l+1)*n) of one array of
 *            ceil(n*levels/64) 64-bit words, LSB first
 *            (wavelet/levelWT/WT.C:54,61,93; wt_int/wt_int_par.hpp:397-398).
 *   nodes  : WTnode records {bitmapPtr, length, parent, leftChild, rightChild}
 *            in heap order, with 4-byte (uintT) or 8-byte (-DLONG) fields and
 *            UINT_T_MAX for absent links (wavelet/levelWT/WT.h:30-35).  Node
 *            records the reference never writes are zero here.
 *   rank   : rank_support_v<1> m_basic_block, ((capacity>>9)+1)*2 words, with
 *            capacity = the bit count rounded up to a multiple of 64
 *            (rank/rank_support_v_par.hpp:78-113).
 *   select : select_support_mcl<t_b> as three flat arrays:
 *            sb_words = the int_vector<0> data of m_superblock (width logn);
 *            desc[i]  = (pool_word_offset << 8) | (is_long << 7) | width for
 *                       superblock i;
 *            pool     = the int_vector<0> data of each superblock's mini block
 *                       (64 entries) or long block (4096 entries), in order
 *            (select/select_support_mcl_par.hpp:83-90,483-561).
 *            info[8]  = size, arg_cnt, logn, logn4, nsb, has_long, sb_nwords,
 *                       pool_nwords (has_long: m_longsuperblock != nullptr).
 */
#ifndef WTG_H
#define WTG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WTG_OK 0
#define WTG_ERR_INVALID 1   /* bad argument */
#define WTG_ERR_OOM 2       /* device allocation failed */
#define WTG_ERR_CUDA 3      /* CUDA runtime error (including: no GPU) */
#define WTG_ERR_TIMEOUT 4   /* a bounded device-side wait gave up; results invalid */
#define WTG_ERR_RANGE 5     /* symbol or index outside the structure */

/* build flags */
#define WTG_RANK 1u     /* rank_support_v<1> over the (concatenated) bitvector */
#define WTG_SELECT1 2u  /* select_support_mcl<1> */
#define WTG_SELECT0 4u  /* select_support_mcl<0> */
#define WTG_ALL 7u

typedef struct wtg_tree wtg_tree; /* wavelet tree + supports, owns device memory */
typedef struct wtg_bv wtg_bv;     /* rank/select supports over a caller bitvector */
typedef struct wtg_lsel wtg_lsel; /* learned select index over a tree's levels */
typedef struct wtg_batch wtg_batch; /* batched builds of many short texts */
typedef struct wtg_huff wtg_huff;   /* Huffman-shaped wavelet tree of a byte text */

const char* wtg_last_error(void);
int wtg_version(void);
/* Number of kernel launches issued by this process so far (all entry points). */
uint64_t wtg_launch_count(void);

/* ------------------------------------------------------------ tree build
 * Replaces WT(symbol* s, uintT n, uintT sigma) (wavelet/levelWT/WT.h:43,
 * levelWT/WT.C:43-227; same contract in ddWT/recWT/serialWT) and the
 * sdsl::wt_int<> constructor (wt_int/wt_int_par.hpp:368-406) with its
 * util::init_support calls for rank and select (:402-404).
 *   seq        : n symbols of elem_bytes (1, 2, 4 or 8) bytes, host memory
 *   levels     : tree height; symbols are read through their low `levels`
 *                bits, bit (levels-1-l) at level l (levelWT/WT.C:62,
 *                wt_int_par.hpp:173).  levels = max(1, log2Up(sigma)) gives
 *                levelWT's tree; 0 derives wt_int's hi(max(1,max symbol))+1
 *                (wt_int_par.hpp:385-395).  1..24 supported.
 *   flags      : WTG_RANK | WTG_SELECT1 | WTG_SELECT0 supports to build over
 *                the concatenated bitvector.
 * The input is copied to the device inside the call. */
int wtg_tree_build(const void* seq, uint64_t n, int elem_bytes, int levels, uint32_t flags,
                   wtg_tree** out);

/* When *out is non-NULL on entry, wtg_tree_build rebuilds that handle in place
 * (reusing its device buffers) instead of creating a new one. */

/* Same as wtg_tree_build, and copies the level bitvector (bit words) and the
 * rank table (rank words, see wtg_tree_info) to host memory while the build
 * runs: the bits of each level leave as soon as its pass is done, and the
 * rank entries of each level as soon as the rank/select pass has covered it
 * (n % 512 == 0 and a page-locked rank_dst; otherwise the whole rank table
 * beside the select finishing kernels).  A page-locked input of at least
 * 2^22 symbols is copied in eight pieces, and the build's first pass counts
 * each piece as it lands.  Either destination may be
 * NULL; levels must be given (not 0).  With page-locked destinations the
 * copies overlap the kernels; pageable ones work but wait for each copy.
 * Returns once the build and the copies are complete.  No counterpart in the
 * reference: WT()'s output arrays (wavelet/levelWT/WT.h:43) filled in place. */
int wtg_tree_build_out(const void* seq, uint64_t n, int elem_bytes, int levels, uint32_t flags, uint64_t* bits_dst,
                       uint64_t* rank_dst, wtg_tree** out);

/* Same, from device memory, enqueued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream).  When *out is non-NULL the handle is rebuilt in
 * place, reusing its device buffers.  Returns once the work is enqueued and
 * the output sizes are known; call wtg_tree_sync() before trusting results. */
int wtg_tree_build_device(const void* d_seq, uint64_t n, int elem_bytes, int levels, uint32_t flags,
                          void* stream, wtg_tree** out);

/* Waits for the handle's stream and reports device-side failures
 * (WTG_ERR_TIMEOUT when a bounded wait expired). */
int wtg_tree_sync(wtg_tree* t);
int wtg_tree_free(wtg_tree* t);

/* n, levels, bit words, rank words */
int wtg_tree_info(wtg_tree* t, uint64_t info[4]);
/* select info[8] (see above) for t_b in {0,1} */
int wtg_tree_select_info(wtg_tree* t, int t_b, uint64_t info[8]);

/* ------------------------------------------------------- tree outputs
 * Host destinations; sizes must match wtg_tree_info / wtg_tree_select_info. */
int wtg_tree_get_bits(wtg_tree* t, uint64_t* dst, uint64_t nwords);
/* WTnode records for heap ids [0, n_entries) with index_bytes (4 or 8) per
 * field: the reference's 2*sigma-entry node array (levelWT/WT.C:46). */
int wtg_tree_get_nodes(wtg_tree* t, int index_bytes, uint64_t n_entries, void* dst);
int wtg_tree_get_rank(wtg_tree* t, uint64_t* dst, uint64_t nwords);
int wtg_tree_get_select(wtg_tree* t, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool);
/* Device pointers of the outputs (valid until the next rebuild or free):
 * ptrs[0]=bits, [1]=rank, [2]=select1 sb_words, [3]=select1 desc,
 * [4]=select1 pool, [5..7]=the same for select0. */
int wtg_tree_device_ptrs(wtg_tree* t, uint64_t ptrs[8]);

/* ------------------------------------------------------------ queries
 * Batched wt_int queries (wt_int/wt_int_par.hpp:519-660), one answer per
 * query.  Host arrays; the _device variants take device arrays and a stream. */
/* operator[](i) (wt_int_par.hpp:519-541) */
int wtg_query_access(wtg_tree* t, const uint64_t* idx, uint64_t nq, uint64_t* out);
/* rank(i, c): occurrences of c in [0, i) (wt_int_par.hpp:553-577) */
int wtg_query_rank(wtg_tree* t, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out);
/* inverse_select(i) -> (rank, symbol) (wt_int_par.hpp:588-611) */
int wtg_query_inverse_select(wtg_tree* t, const uint64_t* idx, uint64_t nq, uint64_t* rank_out,
                             uint64_t* sym_out);
/* select(i, c): position of the i-th c (1-based i); UINT64_MAX where c occurs
 * fewer than i times (the reference throws std::logic_error,
 * wt_int_par.hpp:644-646).  Needs WTG_RANK|WTG_SELECT1|WTG_SELECT0. */
int wtg_query_select(wtg_tree* t, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out);
int wtg_query_access_device(wtg_tree* t, const uint64_t* d_idx, uint64_t nq, uint64_t* d_out, void* stream);
int wtg_query_rank_device(wtg_tree* t, const uint64_t* d_idx, const uint64_t* d_sym, uint64_t nq,
                          uint64_t* d_out, void* stream);

/* ------------------------------------------------------- range queries
 * wt_int's range queries (wt_int/wt_int_par.hpp:684-1048), batched.  A
 * query whose bounds leave the sequence (i > j, j > n, or rb >= n with
 * lb <= rb) answers UINT64_MAX in every field (the reference's precondition).
 * Variable-size answers are written for all queries back to back, query q's
 * first answer after the answers of queries 0..q-1 (counts from the same
 * call, UINT64_MAX read as 0); only the first `cap` answers are stored.  All
 * need a tree built with WTG_RANK. */
/* lex_count(i, j, c) -> (rank(i, c), symbols < c in [i, j), symbols > c in
 * [i, j)) (wt_int_par.hpp:715-745); c >= 2^levels gives (0, j - i, 0) */
int wtg_query_lex_count(wtg_tree* t, const uint64_t* i, const uint64_t* j, const uint64_t* c, uint64_t nq,
                        uint64_t* rank_out, uint64_t* smaller_out, uint64_t* greater_out);
/* lex_smaller_count(i, c) -> (rank(i, c), symbols < c in [0, i))
 * (wt_int_par.hpp:758-782) */
int wtg_query_lex_smaller_count(wtg_tree* t, const uint64_t* i, const uint64_t* c, uint64_t nq,
                                uint64_t* rank_out, uint64_t* smaller_out);
/* range_search_2d(lb, rb, vlb, vrb, report) (wt_int_par.hpp:801-871): the
 * positions p in [lb, rb] (inclusive) with value in [vlb, vrb] (vrb clamped
 * to 2^levels).  count_out gets each query's count; with pos_out / val_out
 * (report; needs WTG_SELECT1|WTG_SELECT0 too) the points (position, value)
 * in the reference's order: values increasing, positions increasing. */
int wtg_query_range_search_2d(wtg_tree* t, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                              const uint64_t* vrb, uint64_t nq, uint64_t* count_out, uint64_t cap,
                              uint64_t* pos_out, uint64_t* val_out);
/* interval_symbols(i, j) (wt_int_par.hpp:684-702): k_out gets the number of
 * distinct symbols of [i, j); with cs_out / rank_i_out / rank_j_out, per
 * symbol in increasing order (c, rank(i, c), rank(j, c)). */
int wtg_query_interval_symbols(wtg_tree* t, const uint64_t* i, const uint64_t* j, uint64_t nq, uint64_t* k_out,
                               uint64_t cap, uint64_t* cs_out, uint64_t* rank_i_out, uint64_t* rank_j_out);
/* expand(v) (wt_int_par.hpp:966-984) for nn nodes v = (offset, size, level,
 * sym), 4 words each: left and right children in the same form (UINT64_MAX
 * fields for a leaf or a node reaching past the bits) */
int wtg_query_expand(wtg_tree* t, const uint64_t* nodes, uint64_t nn, uint64_t* left, uint64_t* right);
/* expand(v, ranges) (wt_int_par.hpp:1027-1048): nr closed ranges [s, e]
 * (2 words each) of node v mapped to its children, in the reference's
 * unsigned 64-bit arithmetic (an empty range is e = s - 1) */
int wtg_query_expand_ranges(wtg_tree* t, const uint64_t v[4], const uint64_t* ranges, uint64_t nr, uint64_t* left,
                            uint64_t* right);
int wtg_query_lex_count_device(wtg_tree* t, const uint64_t* d_i, const uint64_t* d_j, const uint64_t* d_c,
                               uint64_t nq, uint64_t* d_rank, uint64_t* d_smaller, uint64_t* d_greater,
                               void* stream);
int wtg_query_range_count_device(wtg_tree* t, const uint64_t* d_lb, const uint64_t* d_rb, const uint64_t* d_vlb,
                                 const uint64_t* d_vrb, uint64_t nq, uint64_t* d_count, void* stream);

/* --------------------------------------------- standalone bitvector supports
 * rank_support_v<1> (rank/rank_support_v_par.hpp:69-123) and
 * select_support_mcl<1>/<0> (select/select_support_mcl_par.hpp:120-129,
 * 483-561) over the first size_bits bits of a caller bitvector. */
int wtg_bv_build(const uint64_t* words, uint64_t size_bits, uint32_t flags, wtg_bv** out);
int wtg_bv_build_device(const uint64_t* d_words, uint64_t size_bits, uint32_t flags, void* stream,
                        wtg_bv** out);
int wtg_bv_sync(wtg_bv* b);
int wtg_bv_free(wtg_bv* b);
int wtg_bv_rank_words(wtg_bv* b, uint64_t* nwords);
int wtg_bv_get_rank(wtg_bv* b, uint64_t* dst, uint64_t nwords);
int wtg_bv_select_info(wtg_bv* b, int t_b, uint64_t info[8]);
int wtg_bv_get_select(wtg_bv* b, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool);
/* rank_support_v::rank(idx) (rank_support_v_par.hpp:131-142), idx <= size */
int wtg_bv_rank(wtg_bv* b, const uint64_t* idx, uint64_t nq, uint64_t* out);
/* select_support_mcl::select(i) (select_support_mcl_par.hpp:564-611), 1 <= i <= args */
int wtg_bv_select(wtg_bv* b, int t_b, const uint64_t* i, uint64_t nq, uint64_t* out);
int wtg_bv_select_device(wtg_bv* b, int t_b, const uint64_t* d_i, uint64_t nq, uint64_t* d_out,
                         void* stream);

/* Allocation-free rank table build.  No counterpart in the reference: an
 * addition for callers that cannot allocate device memory -- code that runs
 * inside a memory budget owned by another framework, or in a phase where a
 * cudaMalloc would synchronise the device or is forbidden by the pool in use.
 * Builds the same rank_support_v<1> table as wtg_bv_build (WTG_RANK) from
 * d_words (size_bits bits, device memory) into d_rank (device memory of
 * 2*(floor(ceil(size_bits/64)/8)+1) words, the size wtg_bv_rank_words gives),
 * on `stream`; the calling thread then waits for that stream (not for the
 * whole device) to read the pass's error word.  It calls no
 * cudaMalloc/cudaFree: its scratch is one fixed device array inside the
 * library (about 1 MB, held on every GPU that loads the library until exit),
 * which limits size_bits to 2^34; larger inputs return WTG_ERR_RANGE.  The
 * first call on a device looks up that array's device address (make it
 * before any stream capture); the address is kept until the process exits,
 * so the entry point must not be used after a cudaDeviceReset.  All calls
 * share the array, so calls that overlap on the GPU (other threads or
 * streams) race. */
int wtg_rank_build_noalloc(const uint64_t* d_words, uint64_t size_bits, uint64_t* d_rank, void* stream);

/* ------------------------------------------------------------ batched builds
 * Many independent texts, each with its own wavelet tree, rank_support_v<1>
 * and select_support_mcl<1>/<0> -- what a loop of WT() calls
 * (wavelet/levelWT/WT.h:43) or of wt_int constructions
 * (wt_int/wt_int_par.hpp:368-406) plus init_support would give, one text per
 * call -- built in one persistent launch that pulls work items from a
 * device queue, replayed from a CUDA graph after the first run.  A text of
 * at most `whole_max` symbols is one item, built by one CTA from histogram
 * to select tables; a longer text is split into (text, tile) key
 * histograms, (text, tile) level bits of every level, (text, rank tile)
 * rank_support_v entries and select samples, and (text) select_support_mcl
 * finishing, each waiting for its text's previous phase.
 *   lengths : symbols of each text (ntexts entries); texts are u8 symbols
 *             read through their low `levels` bits, concatenated in order
 *   levels  : 1..4
 *   flags   : WTG_RANK | WTG_SELECT1 | WTG_SELECT0 (select implies rank)
 *   stream  : the stream the batch runs on (NULL: the batch makes its own)
 * The plan allocates every output region (sizes follow from the lengths).
 * The first wtg_batch_run times the candidate shapes (symbols per thread of
 * the level pass x split tile and whole-text bound) on the loaded input,
 * keeps the fastest and captures the build in a CUDA graph; later runs
 * replay the graph.  Per-text outputs have the
 * single-sequence layouts (wtg_tree_get_bits / _get_rank / _get_select of a
 * tree built with the same levels). */
int wtg_batch_plan(const uint64_t* lengths, uint64_t ntexts, int levels, uint32_t flags, void* stream,
                   wtg_batch** out);
/* device address and size of the input buffer (the concatenated texts) */
int wtg_batch_input(wtg_batch* b, void** d_input, uint64_t* nbytes);
/* copy the concatenated texts from host memory into the input buffer */
int wtg_batch_load(wtg_batch* b, const void* texts);
int wtg_batch_run(wtg_batch* b);
/* fix the shape instead of timing the candidates on the first run:
 * `tile` symbols per split-text tile (a multiple of 256 x
 * symbols_per_thread, up to 2^24), the longest text built whole by one CTA
 * (-1: the total symbols over the resident CTAs, at least 65536; 0: every
 * text split) and the level pass's symbols per thread (32, or 64 for 1-2
 * levels) */
int wtg_batch_set_shape(wtg_batch* b, int tile, int64_t whole_max, int symbols_per_thread);
int wtg_batch_sync(wtg_batch* b);
int wtg_batch_free(wtg_batch* b);
/* after wtg_batch_sync.  text info: n, levels, bit words, rank words, ones,
 * zeros, symbols per split tile, and 1 if the text was built whole */
int wtg_batch_text_info(wtg_batch* b, uint64_t t, uint64_t info[8]);
/* select info[8] of text t, as wtg_tree_select_info */
int wtg_batch_select_info(wtg_batch* b, uint64_t t, int t_b, uint64_t info[8]);
int wtg_batch_get_bits(wtg_batch* b, uint64_t t, uint64_t* dst, uint64_t nwords);
int wtg_batch_get_rank(wtg_batch* b, uint64_t t, uint64_t* dst, uint64_t nwords);
int wtg_batch_get_select(wtg_batch* b, uint64_t t, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool);
/* after a run: the shape in use (split tile, whole-text bound, symbols per
 * thread), how many texts were built whole, and the first run's time of each
 * candidate shape in ms (0: not tried; all 0 after wtg_batch_set_shape) */
int wtg_batch_shape(wtg_batch* b, int* tile, int64_t* whole_max, int* symbols_per_thread, uint64_t* whole_texts,
                    float ms[8]);

/* ------------------------------------------------- suffix array and BWT
 * The first two steps of the reference's FM-index construction
 * (fm-index/par/WT.C:33-41): SA = divsufsort(s) (suffixArray/divsufsort,
 * 32-bit entries, no sentinel: a suffix that is a prefix of another sorts
 * first) and bwt[i] = s[SA[i] - 1], or s[n - 1] where SA[i] = 0.  Computed
 * on the GPU by prefix doubling over radix sorts; identical to divsufsort's
 * array.  n < 2^31. */
int wtg_suffix_array(const uint8_t* text, uint64_t n, int32_t* sa_out);
/* SA and BWT in one call; either output may be NULL (not both) */
int wtg_bwt(const uint8_t* text, uint64_t n, uint8_t* bwt_out, int32_t* sa_out);
/* device text / outputs on a stream (d_sa or d_bwt may be NULL); returns
 * once the stream has finished; rounds (may be NULL) gets the number of
 * doubling rounds.  Allocates its scratch (about 33 bytes per symbol). */
int wtg_suffix_array_device(const uint8_t* d_text, uint64_t n, int32_t* d_sa, uint8_t* d_bwt, void* stream,
                            int* rounds);

/* ------------------------------------------------------------ FM-index count
 * Backward search over a tree built (with WTG_RANK) on the BWT of a text,
 * its symbols coded 0..sigma-1: the reference's FM-index is the wavelet tree
 * of s[SA[i]-1] (s[n-1] where SA[i] == 0) with SA from divsufsort
 * (fm-index/par/WT.C:33-45); the reference stops at construction, and this
 * adds the count query.  C[c] = number of BWT symbols below c (sigma
 * entries).  Pattern p is pat[off[p] .. off[p+1]) (byte codes); out[p] is
 * the size of its suffix-array range, i.e. its number of occurrences.  A
 * code >= sigma gives 0, an empty pattern gives n.  sigma <= 256. */
int wtg_fm_count(wtg_tree* t, const uint64_t* C, uint64_t sigma, const uint8_t* pat, const uint64_t* off,
                 uint64_t npat, uint64_t* out);
int wtg_fm_count_device(wtg_tree* t, const uint64_t* d_C, uint64_t sigma, const uint8_t* d_pat,
                        const uint64_t* d_off, uint64_t npat, uint64_t* d_out, void* stream);

/* ------------------------------------------ per-level and learned select
 * A query is a pair (level, k): the position, inside level `level` of the
 * tree, of that level's k-th one (t_b = 1) or zero (t_b = 0), k >= 1;
 * UINT64_MAX where the level holds fewer than k.  Levels are the n-bit
 * slices of the concatenated bitvector.
 *
 * wtg_tree_level_select is the plain route: select_support_mcl<t_b> on the
 * concatenated bitvector after adding the args before the level, which is
 * wt_int's per-level select step (wt_int/wt_int_par.hpp:651-656) with the
 * whole level as the node.  Needs WTG_ALL. */
int wtg_tree_level_select(wtg_tree* t, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                          uint64_t* out);
int wtg_tree_level_select_device(wtg_tree* t, int t_b, const uint64_t* d_level, const uint64_t* d_k, uint64_t nq,
                                 uint64_t* d_out, void* stream);

/* Learned select index beside select_support_mcl.  No counterpart in the
 * reference.  Per level and polarity, the args are cut into at most
 * `segments` segments of 2^g args; each gets a line fitted on the GPU by
 * least squares to `samples` (k, select(k)) pairs taken from the plain
 * select, and an error window that holds for every k of the segment.  A
 * query predicts the position and searches the window exactly through a
 * rank directory of the superblocks (per 8192 bits the ones before them,
 * per 512-bit superblock an int8 residual against the line between: 24
 * bytes per 8192 bits, small enough to stay in L2), then reads the
 * superblock's one 64-byte line; segments whose window exceeds max_window
 * positions, and blocks whose residuals overflow int8, are answered by the
 * plain select.  Answers equal
 * wtg_tree_level_select's.  The index reads the tree's bitvector, rank and
 * select tables: it is valid until the tree is rebuilt or freed (queries
 * after a rebuild return WTG_ERR_INVALID).  Needs a tree built with WTG_ALL.
 * Builds on the tree's stream and waits for it. */
int wtg_lsel_build(wtg_tree* t, uint32_t segments, uint32_t samples, uint32_t max_window, wtg_lsel** out);
int wtg_lsel_free(wtg_lsel* m);
/* info[8]: segments (both polarities), index bytes (segment records and
 * the rank directory), segments answered by the plain select, largest
 * window of the others, sum of their windows, searches that fell back since
 * the build (0 unless the tables are inconsistent), segments and samples
 * parameters */
int wtg_lsel_info(wtg_lsel* m, uint64_t info[8]);
/* one level's model: lvl_info = {args before the level, args in it, g,
 * segments}; rec (may be NULL) receives 4 u32 per segment: base, slope
 * (16.16 fixed), dlo, dhi (int32) */
int wtg_lsel_get_level(wtg_lsel* m, int t_b, int level, uint64_t lvl_info[4], uint32_t* rec, uint64_t nseg);
int wtg_lsel_query(wtg_lsel* m, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq, uint64_t* out);
int wtg_lsel_query_device(wtg_lsel* m, int t_b, const uint64_t* d_level, const uint64_t* d_k, uint64_t nq,
                          uint64_t* d_out, void* stream);

/* ------------------------------------------------------------ profiling
 * When enabled, every build records a CUDA event pair around each kernel it
 * launches, on the launching stream.  wtg_profile_read waits for those events
 * and returns, per kernel class, the number of launches and their summed
 * device time in ms, then clears the record.  Classes: 0 level pass with
 * partition, 1 last level pass, 2 key histogram, 3 node tables and scans,
 * 4 bitvector pass (rank + select samples), 5 select finishing kernels. */
#define WTG_PROF_CLASSES 6
int wtg_profile_enable(int on);
int wtg_profile_read(uint64_t launches[WTG_PROF_CLASSES], double ms[WTG_PROF_CLASSES]);

/* ------------------------------------------- Huffman-shaped wavelet tree
 * sdsl::wt_huff<> over a byte text (wt_huff/wt_huff_par.hpp, built as
 * wt_huff/wt_pc_par.hpp:321-361 builds it), the tree of the reference's
 * FM-index (fm-index/par/WT.C:44).  Shape: Huffman code of the byte counts,
 * ties broken by (frequency, node number) with leaves numbered by byte value
 * and merged nodes after them (wt_huff_par.hpp:82-117); nodes in breadth-first
 * order, each inner node's bitvector at bv_pos = the sizes of the inner nodes
 * before it; rank_support_v<1> / select_support_mcl over the concatenated
 * bitvector as flags ask (select implies rank).
 *   info[5]  : n, sigma, bitvector bits, tree nodes, rank table words
 *   get_tree : per node (bv_pos, bv_pos_rank -- the ones before bv_pos, or a
 *              leaf's byte --, parent, child0, child1), 0xFFFF for none, 5
 *              words each; per byte its leaf (0xFFFF: absent) and path (bit d
 *              set when the (d+1)-th edge goes right, length << 56)
 *   access / rank / select / inverse_select: wt_pc's operator[], rank(i, c),
 *              select(i, c), inverse_select(i) (wt_huff/wt_pc_par.hpp:430-552);
 *              select gives n for a byte not in the text and UINT64_MAX for i
 *              beyond its occurrences (the reference asserts)
 *   fm_count : backward search over a BWT's tree, C[256] = bytes below c */
int wtg_huff_build(const uint8_t* text, uint64_t n, uint32_t flags, wtg_huff** out);
int wtg_huff_build_device(const uint8_t* d_text, uint64_t n, uint32_t flags, void* stream, wtg_huff** out);
int wtg_huff_free(wtg_huff* h);
int wtg_huff_info(wtg_huff* h, uint64_t info[5]);
int wtg_huff_get_bits(wtg_huff* h, uint64_t* dst, uint64_t nwords);
int wtg_huff_get_tree(wtg_huff* h, uint64_t* nodes, uint64_t* leaves, uint64_t* paths);
int wtg_huff_get_rank(wtg_huff* h, uint64_t* dst, uint64_t nwords);
int wtg_huff_select_info(wtg_huff* h, int t_b, uint64_t info[8]);
int wtg_huff_get_select(wtg_huff* h, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool);
int wtg_huff_access(wtg_huff* h, const uint64_t* idx, uint64_t nq, uint64_t* out);
int wtg_huff_rank(wtg_huff* h, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out);
int wtg_huff_select(wtg_huff* h, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out);
int wtg_huff_inverse_select(wtg_huff* h, const uint64_t* idx, uint64_t nq, uint64_t* rank_out, uint64_t* sym_out);
int wtg_huff_fm_count(wtg_huff* h, const uint64_t* C, const uint8_t* pat, const uint64_t* off, uint64_t npat,
                      uint64_t* out);
/* the same on device arrays, enqueued on `stream` (offsets must not
 * decrease; they are not checked on the host) */
int wtg_huff_fm_count_device(wtg_huff* h, const uint64_t* d_C, const uint8_t* d_pat, const uint64_t* d_off,
                             uint64_t npat, uint64_t* d_out, void* stream);

/* ---------------------------------------------- sdsl serialize() streams
 * The byte streams sdsl's serialize() writes (what sdsl::store_to_file puts
 * in a file), so that sdsl consumers load GPU-built structures with their
 * own load(), and so that outputs compare byte for byte as the reference's
 * own check does (wt_int/compareResults.py:1-15).
 * wtg_tree_serialize: wt_int<>::serialize (wt_int/wt_int_par.hpp:887-899):
 *   size (u64), sigma (u64, the non-empty leaves), the level bit_vector, the
 *   rank_support_v, select_support_mcl<1>, select_support_mcl<0>, max_level
 *   (u32) -- needs a tree built with WTG_ALL.
 * wtg_bv_serialize: part WTG_RANK gives rank_support_v<1>::serialize
 *   (rank/rank_support_v_par.hpp:154-164), WTG_SELECT1 / WTG_SELECT0
 *   select_support_mcl<1/0>::serialize (select/select_support_mcl_par.hpp:
 *   644-681).
 * Each int_vector inside is its size in bits (u64), its width (one byte, for
 * run-time widths only) and its ceil(bits/64) words.  With dst == NULL only
 * *len is set; otherwise dst (host memory) must hold cap >= *len bytes.
 * wtg_tree_sigma: wt_int's sigma, the number of non-empty leaves. */
int wtg_tree_serialize(wtg_tree* t, void* dst, uint64_t cap, uint64_t* len);
int wtg_tree_sigma(wtg_tree* t, uint64_t* sigma);
int wtg_bv_serialize(wtg_bv* b, uint32_t part, void* dst, uint64_t cap, uint64_t* len);

/* ----------------------------------------------- failure handling knobs
 * No counterpart in the reference (its CPU code has no device waits; its
 * error sites throw std::logic_error, wt_int/wt_int_par.hpp:377,645).
 *
 * Every device-side wait of the builds is bounded: a decoupled look-back
 * spins at most `lookback_spins` times (with a backoff of up to 1 us each,
 * default 2^22: seconds), an mbarrier wait tries at most `mbarrier_tries`
 * times (default 2^24).  On expiry the kernel records the failure and
 * returns, and the build's sync reports WTG_ERR_TIMEOUT; the context stays
 * usable.  wtg_set_wait_limits changes both limits for later launches on the
 * current device (0 restores a default).
 *
 * Test hooks, host side only (they never make a device fault):
 * wtg_test_fail_alloc(k), k >= 1, makes the k-th next device allocation of
 * the library fail with WTG_ERR_OOM (0 disarms); wtg_test_stall_lookback(1)
 * makes the next rank/select pass over a caller bitvector start its tile
 * counter at 1, so tile 0 never publishes its count and the other tiles'
 * look-back waits run out (WTG_ERR_TIMEOUT). */
int wtg_set_wait_limits(uint32_t lookback_spins, uint32_t mbarrier_tries);
int wtg_test_fail_alloc(int64_t nth);
int wtg_test_stall_lookback(int on);

/* --------------------------------------------------------------- helpers */
/* Alphabet remap of levelWT/WTTime.C:80-94: every symbol becomes its rank
 * among the distinct values present; *sigma_out = number of distinct values.
 * In place on host memory. */
int wtg_remap_alphabet(void* seq, uint64_t n, int elem_bytes, uint64_t* sigma_out);

#ifdef __cplusplus
}
#endif
#endif
