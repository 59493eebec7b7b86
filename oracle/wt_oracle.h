/*
 * wt_oracle.h -- CPU restatement of the reference's wavelet-tree build,
 * rank_support_v, select_support_mcl and wt_int query algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, the
 * smoke entry and the CPU-baseline leg of the benchmark call it to produce
 * expected outputs and CPU timings.  The product (libwtg) never links or
 * calls it, and the product has no CPU fallback.
 *
 * Every function names the reference file:line it restates (paths are
 * relative to the jlabeit/wavelet-suffix-fm-index source tree).
 */
#ifndef WT_ORACLE_H
#define WT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One wavelet-tree node with 64-bit fields (WTnode, wavelet/levelWT/WT.h:30-35).
 * UINT64_MAX marks an absent parent/child (UINT_T_MAX in the reference). */
typedef struct {
  uint64_t bitmapPtr, length, parent, leftChild, rightChild;
} or_node;

/* utils::log2Up (wavelet/levelWT/utils.h:55-60). */
int or_log2_up(uint64_t i);
/* sdsl bits::hi: position of the most significant set bit, 0 for x == 0. */
int or_hi(uint64_t x);
/* levels = max(1, log2Up(sigma)) (wavelet/levelWT/WT.C:53). */
int or_levels_for_sigma(uint64_t sigma);

/* levelWT WT() (wavelet/levelWT/WT.C:43-227).  Symbols are elem_bytes wide
 * (1, 2, 4 or 8); the tree has `levels` levels over codes [0, 2^levels).
 * wt receives ceil(n*levels/64) words (level l at bits [l*n,(l+1)*n), LSB
 * first).  nodes (may be NULL) receives n_nodes entries in heap order; entries
 * the build never visits are zeroed (the reference leaves them uninitialised).
 * Uses OpenMP when compiled with it.  Returns 0 on success. */
int or_wt_levelwt(const void* s, int elem_bytes, uint64_t n, int levels,
                  uint64_t* wt, or_node* nodes, uint64_t n_nodes);

/* serialWT WT() (wavelet/serialWT/WT.C:32-103): the serial level-by-level
 * build, used to cross-check or_wt_levelwt. */
int or_wt_serial(const void* s, int elem_bytes, uint64_t n, int levels,
                 uint64_t* wt, or_node* nodes, uint64_t n_nodes);

/* Alphabet remap of levelWT/WTTime.C:80-94: replaces each symbol by its rank
 * among the distinct values present (ascending).  Returns sigma. */
uint64_t or_remap_alphabet(void* s, int elem_bytes, uint64_t n);

/* rank_support_v<1> table (rank/rank_support_v_par.hpp:69-123).
 * Table has or_rank_words(size) words. */
uint64_t or_rank_words(uint64_t size_bits);
void or_rank_build(const uint64_t* data, uint64_t size_bits, uint64_t* table);
/* rank_support_v::rank (rank/rank_support_v_par.hpp:131-142). */
uint64_t or_rank1(const uint64_t* table, const uint64_t* data, uint64_t idx);

/* select_support_mcl<t_b> (select/select_support_mcl_par.hpp).  The handle
 * holds the structure in a flat, packed form:
 *   sb_words : the int_vector<0> data of m_superblock (width logn)
 *   desc[i]  : (pool word offset << 8) | (is_long << 7) | width
 *   pool     : int_vector<0> data of every mini (64 entries) or long (4096
 *              entries) block, concatenated in superblock order.
 * info[0..7] = size, arg_cnt, logn, logn4, nsb, has_long, sb_nwords, pool_nwords.
 * use_rule: 0 = reference rule (init_slow when size < 100000, else init_fast),
 *           1 = force init_slow, 2 = force init_fast. */
typedef struct or_select or_select;
or_select* or_select_new(const uint64_t* data, uint64_t size_bits, int t_b, int use_rule);
void or_select_info(const or_select* h, uint64_t info[8]);
void or_select_copy(const or_select* h, uint64_t* sb_words, uint64_t* desc, uint64_t* pool);
/* select(i), 1 <= i <= arg_cnt (select/select_support_mcl_par.hpp:564-611). */
uint64_t or_select_query(const or_select* h, const uint64_t* data, uint64_t i);
void or_select_free(or_select* h);

/* wt_int queries over the concatenated level bitvector (tree), with its
 * rank table and select handles (wt_int/wt_int_par.hpp:519-660). */
uint64_t or_wt_access(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n,
                      int levels, uint64_t i);
uint64_t or_wt_rank(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n,
                    int levels, uint64_t i, uint64_t c);
/* inverse_select: returns rank, writes the symbol to *c_out. */
uint64_t or_wt_inverse_select(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n,
                              int levels, uint64_t i, uint64_t* c_out);
/* select(i, c); returns UINT64_MAX when c does not occur i times (the
 * reference throws std::logic_error, wt_int_par.hpp:645). */
uint64_t or_wt_select(const uint64_t* tree, const uint64_t* rank_tbl,
                      const or_select* sel1, const or_select* sel0,
                      uint64_t n, int levels, uint64_t i, uint64_t c);

/* wt_int's range queries (wt_int_par.hpp:684-1048).  lex_count writes
 * (rank(i, c), smaller, greater), lex_smaller_count (rank(i, c), smaller);
 * range_search_2d returns the point count and, with report, stores the first
 * cap points (position, value) in the reference's order; interval_symbols
 * returns k and stores the first cap (symbol, rank(i, c), rank(j, c));
 * expand maps a node (offset, size, level, sym) to its children, and
 * expand_ranges closed ranges [s, e] of a node to its children's. */
void or_wt_lex_count(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels, uint64_t i,
                     uint64_t j, uint64_t c, uint64_t* out);
void or_wt_lex_smaller_count(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                             uint64_t i, uint64_t c, uint64_t* out);
uint64_t or_wt_range_search_2d(const uint64_t* tree, const uint64_t* rank_tbl, const or_select* sel1,
                               const or_select* sel0, uint64_t n, int levels, uint64_t lb, uint64_t rb,
                               uint64_t vlb, uint64_t vrb, int report, uint64_t cap, uint64_t* pos,
                               uint64_t* val);
uint64_t or_wt_interval_symbols(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                                uint64_t i, uint64_t j, uint64_t cap, uint64_t* cs, uint64_t* rank_i,
                                uint64_t* rank_j);
void or_wt_expand(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, const uint64_t* v, uint64_t* left,
                  uint64_t* right);
void or_wt_expand_ranges(const uint64_t* tree, const uint64_t* rank_tbl, const uint64_t* v,
                         const uint64_t* ranges, uint64_t nr, uint64_t* left, uint64_t* right);

/* Batched query helpers (loop over the scalar functions above, OpenMP). */
void or_wt_access_batch(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                        const uint64_t* idx, uint64_t nq, uint64_t* out);
void or_wt_rank_batch(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                      const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out);
void or_wt_lex_count_batch(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                           const uint64_t* i, const uint64_t* j, const uint64_t* c, uint64_t nq, uint64_t* out);
void or_wt_lex_smaller_count_batch(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                                   const uint64_t* i, const uint64_t* c, uint64_t nq, uint64_t* out);
void or_wt_range_count_batch(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels,
                             const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb, const uint64_t* vrb,
                             uint64_t nq, uint64_t* out);
void or_select_batch(const or_select* h, const uint64_t* data, const uint64_t* q, uint64_t nq,
                     uint64_t* out);

/* FM-index core (fm-index/par/WT.C:33-45): suffix array, BWT, and counting
 * by backward search over the wavelet tree of the BWT. */
/* Suffix array of the n bytes at s: all suffixes, no sentinel, a proper
 * prefix before its extensions -- the array divsufsort returns
 * (fm-index/par/WT.C:35-36).  Prefix doubling; returns 0, or -1 when out of
 * memory. */
int or_suffix_array_u8(const uint8_t* s, int64_t n, int64_t* sa);
/* bwt[i] = s[sa[i] - 1], or s[n - 1] where sa[i] == 0 (fm-index/par/WT.C:38-41) */
void or_bwt_u8(const uint8_t* s, const int64_t* sa, int64_t n, uint8_t* bwt);
/* Backward search: for pattern p (codes pat[off[p] .. off[p+1])), the size
 * of its suffix-array range, from [0, n) narrowed right to left by
 * sp = C[c] + rank(sp, c), ep = C[c] + rank(ep, c) with wt_int's rank over
 * the tree of the BWT codes; C[c] = number of codes below c. */
void or_fm_count(const uint64_t* tree, const uint64_t* rank_tbl, uint64_t n, int levels, const uint64_t* C,
                 uint64_t sigma, const uint8_t* pat, const uint64_t* off, uint64_t npat, uint64_t* out);

/* Number of OpenMP threads the oracle uses (1 without OpenMP). */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
