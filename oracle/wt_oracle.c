/*
 * wt_oracle.c -- CPU restatement of the reference's wavelet-tree build,
 * rank_support_v, select_support_mcl and wt_int queries.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker used by tests/, by the smoke
 * entry and by the benchmark's CPU-baseline leg.  The product never calls it.
 *
 * The sdsl primitives the reference relies on (bit_vector / int_vector<0>
 * packing, bits::cnt/sel/hi, the rank/select traits) are restated here from
 * their documented behaviour; sdsl itself is not part of the reference tree.
 */
#include "wt_oracle.h"
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_NONE UINT64_MAX
#define OR_THRESHOLD 10000 /* wavelet/levelWT/WT.C:29 */

typedef struct { uint64_t start, length, nodeID, zc; } or_chunk;

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline void or_word(uint64_t* w, uint64_t v) {
  if (v) __atomic_fetch_or(w, v, __ATOMIC_RELAXED); /* writeOr, WT.C:31-35 */
}

static inline int popc(uint64_t x) { return __builtin_popcountll(x); }

/* bits::sel: position of the i-th (1-based) set bit of x. */
static inline int sel64(uint64_t x, uint64_t i) {
  for (uint64_t k = 1; k < i; k++) x &= x - 1;
  return __builtin_ctzll(x);
}

int or_log2_up(uint64_t i) {
  int a = 0;
  uint64_t b = i - 1;
  while (b > 0) { b >>= 1; a++; }
  return a;
}

int or_hi(uint64_t x) { return x == 0 ? 0 : 63 - __builtin_clzll(x); }

int or_levels_for_sigma(uint64_t sigma) {
  int l = or_log2_up(sigma);
  return l < 1 ? 1 : l;
}

/* ---------------------------------------------------------------- levelWT */

#define OR_T uint8_t
#define OR_SUF u8
#include "wt_oracle_level.inc"
#undef OR_T
#undef OR_SUF
#define OR_T uint16_t
#define OR_SUF u16
#include "wt_oracle_level.inc"
#undef OR_T
#undef OR_SUF
#define OR_T uint32_t
#define OR_SUF u32
#include "wt_oracle_level.inc"
#undef OR_T
#undef OR_SUF
#define OR_T uint64_t
#define OR_SUF u64
#include "wt_oracle_level.inc"
#undef OR_T
#undef OR_SUF

int or_wt_levelwt(const void* s, int eb, uint64_t n, int levels, uint64_t* wt, or_node* nodes,
                  uint64_t n_nodes) {
  if (levels < 1 || levels > 64) return -2;
  switch (eb) {
    case 1: return levelwt_u8((const uint8_t*)s, n, levels, wt, nodes, n_nodes);
    case 2: return levelwt_u16((const uint16_t*)s, n, levels, wt, nodes, n_nodes);
    case 4: return levelwt_u32((const uint32_t*)s, n, levels, wt, nodes, n_nodes);
    case 8: return levelwt_u64((const uint64_t*)s, n, levels, wt, nodes, n_nodes);
    default: return -2;
  }
}

static inline uint64_t ld_sym(const void* s, int eb, uint64_t i) {
  switch (eb) {
    case 1: return ((const uint8_t*)s)[i];
    case 2: return ((const uint16_t*)s)[i];
    case 4: return ((const uint32_t*)s)[i];
    default: return ((const uint64_t*)s)[i];
  }
}
static inline void st_sym(void* s, int eb, uint64_t i, uint64_t v) {
  switch (eb) {
    case 1: ((uint8_t*)s)[i] = (uint8_t)v; break;
    case 2: ((uint16_t*)s)[i] = (uint16_t)v; break;
    case 4: ((uint32_t*)s)[i] = (uint32_t)v; break;
    default: ((uint64_t*)s)[i] = v; break;
  }
}

/* serialWT (wavelet/serialWT/WT.C:32-103): one sequential sweep per level. */
int or_wt_serial(const void* s, int eb, uint64_t n, int levels, uint64_t* wt, or_node* nodes,
                 uint64_t n_nodes) {
  if (levels < 1 || levels > 64) return -2;
  uint64_t nw = (n * (uint64_t)levels + 63) / 64;
  memset(wt, 0, nw * 8);
  if (nodes && n_nodes) {
    memset(nodes, 0, n_nodes * sizeof(or_node));
    nodes[0].parent = OR_NONE;
  }
  if (n == 0) return 0;
  uint64_t* s1 = (uint64_t*)malloc(n * 8);
  uint64_t* s2 = (uint64_t*)malloc(n * 8);
  uint64_t cap = n + 1;
  if (levels < 40 && (1ull << levels) < cap) cap = 1ull << levels;
  or_chunk* cur = (or_chunk*)malloc(cap * sizeof(or_chunk));
  or_chunk* nxt = (or_chunk*)malloc(cap * sizeof(or_chunk));
  for (uint64_t i = 0; i < n; i++) s1[i] = ld_sym(s, eb, i);
  uint64_t nc = 1;
  cur[0].start = 0; cur[0].length = n; cur[0].nodeID = 0;
  for (int l = 0; l < levels; l++) {
    uint64_t pos = (uint64_t)l * n;
    int bit = levels - l - 1;
    uint64_t nn = 0;
    for (uint64_t j = 0; j < nc; j++) {
      uint64_t start = cur[j].start, len = cur[j].length, id = cur[j].nodeID;
      if (nodes && id < n_nodes) { nodes[id].bitmapPtr = pos; nodes[id].length = len; }
      if (l == levels - 1) {
        for (uint64_t i = start; i < start + len; i++, pos++)
          if ((s1[i] >> bit) & 1) wt[pos / 64] |= 1ull << (pos % 64);
        if (nodes && id < n_nodes) nodes[id].leftChild = nodes[id].rightChild = OR_NONE;
      } else {
        uint64_t left = 0, right = 0;
        for (uint64_t i = start; i < start + len; i++) right += !((s1[i] >> bit) & 1);
        uint64_t zc = right;
        for (uint64_t i = start; i < start + len; i++, pos++) {
          if ((s1[i] >> bit) & 1) { wt[pos / 64] |= 1ull << (pos % 64); s2[start + right++] = s1[i]; }
          else s2[start + left++] = s1[i];
        }
        if (zc) {
          if (nodes && 2 * id + 1 < n_nodes) nodes[2 * id + 1].parent = id;
          if (nodes && id < n_nodes) nodes[id].leftChild = 2 * id + 1;
          nxt[nn].start = start; nxt[nn].length = zc; nxt[nn].nodeID = 2 * id + 1; nn++;
        } else if (nodes && id < n_nodes) nodes[id].leftChild = OR_NONE;
        if (len - zc) {
          if (nodes && 2 * id + 2 < n_nodes) nodes[2 * id + 2].parent = id;
          if (nodes && id < n_nodes) nodes[id].rightChild = 2 * id + 2;
          nxt[nn].start = start + zc; nxt[nn].length = len - zc; nxt[nn].nodeID = 2 * id + 2; nn++;
        } else if (nodes && id < n_nodes) nodes[id].rightChild = OR_NONE;
      }
    }
    or_chunk* t = cur; cur = nxt; nxt = t; nc = nn;
    uint64_t* ts = s1; s1 = s2; s2 = ts;
  }
  free(s1); free(s2); free(cur); free(nxt);
  return 0;
}

/* levelWT/WTTime.C:80-94 */
uint64_t or_remap_alphabet(void* s, int eb, uint64_t n) {
  if (n == 0) return 0;
  uint64_t k = 0;
  for (uint64_t i = 0; i < n; i++) { uint64_t v = ld_sym(s, eb, i); if (v > k) k = v; }
  k += 1;
  uint64_t* A = (uint64_t*)calloc(k + 1, 8);
  for (uint64_t i = 0; i < n; i++) A[ld_sym(s, eb, i)] = 1;
  uint64_t run = 0;
  for (uint64_t v = 0; v <= k; v++) { uint64_t t = A[v]; A[v] = run; run += t; }
  for (uint64_t i = 0; i < n; i++) st_sym(s, eb, i, A[ld_sym(s, eb, i)]);
  free(A);
  return run;
}

/* -------------------------------------------------------- rank_support_v */

uint64_t or_rank_words(uint64_t size) {
  if (size == 0) return 2; /* int_vector<64>(2,0), rank_support_v_par.hpp:74-76 */
  uint64_t cap = (size + 63) / 64 * 64;
  return ((cap >> 9) + 1) << 1; /* rank_support_v_par.hpp:78 */
}

/* rank/rank_support_v_par.hpp:69-123.  The constructor reads data[8*b] for
 * b = capacity>>9, one word past the data when capacity % 512 == 0; sdsl
 * keeps a zero word there, so that word reads as 0 here. */
void or_rank_build(const uint64_t* data, uint64_t size, uint64_t* tbl) {
  if (size == 0) { tbl[0] = tbl[1] = 0; return; }
  uint64_t cap = (size + 63) / 64 * 64;
  uint64_t W = cap >> 6, NB = cap >> 9;
#pragma omp parallel for schedule(static)
  for (int64_t bb = 0; bb <= (int64_t)NB; bb++) {
    uint64_t b = (uint64_t)bb;
    uint64_t w0 = (b << 3) < W ? data[b << 3] : 0;
    uint64_t sum = popc(w0);
    uint64_t second = 0;
    uint64_t end = (b << 3) + 8 < W ? (b << 3) + 8 : W;
    uint64_t i;
    for (i = (b << 3) + 1; i < end; i++) {
      second |= sum << (63 - 9 * (i & 7));
      sum += popc(data[i]);
    }
    if (i % 8 != 0) second |= sum << (63 - 9 * (i & 7));
    tbl[2 * b] = sum;
    tbl[2 * b + 1] = second;
  }
  /* exclusive scan over the even words (rank_support_v_par.hpp:112-113) */
  uint64_t run = 0;
  for (uint64_t b = 0; b <= NB; b++) { uint64_t t = tbl[2 * b]; tbl[2 * b] = run; run += t; }
}

/* rank_support_v_par.hpp:131-142 */
uint64_t or_rank1(const uint64_t* tbl, const uint64_t* data, uint64_t idx) {
  const uint64_t* p = tbl + ((idx >> 8) & 0xFFFFFFFFFFFFFFFEull);
  uint64_t r = p[0] + ((p[1] >> (63 - 9 * ((idx & 0x1FF) >> 6))) & 0x1FF);
  if (idx & 0x3F) r += popc(data[idx >> 6] & ((1ull << (idx & 63)) - 1));
  return r;
}

/* ---------------------------------------------------- select_support_mcl */

struct or_select {
  uint64_t size, arg_cnt, nsb;
  uint32_t logn, logn2, logn4;
  int has_long, t_b;
  uint64_t* sb_start; /* unpacked m_superblock */
  uint64_t* desc;
  uint64_t* sb_words;
  uint64_t sb_nwords;
  uint64_t* pool;
  uint64_t pool_nwords;
};

/* the word as seen by select_support_trait<t_b,1>: ones for t_b=1, zeros
 * (~w) for t_b=0; bits at or past `size` are masked off */
static inline uint64_t arg_word(const uint64_t* data, uint64_t size, uint64_t wi, int t_b) {
  uint64_t w = data[wi];
  if (!t_b) w = ~w;
  uint64_t lo = wi << 6;
  if (lo + 64 > size) {
    uint64_t keep = size - lo;
    w &= keep >= 64 ? ~0ull : ((1ull << keep) - 1);
  }
  return w;
}

static void pack_put(uint64_t* words, uint64_t j, int w, uint64_t v) {
  uint64_t off = j * (uint64_t)w;
  uint64_t wi = off >> 6;
  int sh = (int)(off & 63);
  if (w < 64) v &= (1ull << w) - 1;
  words[wi] |= v << sh;
  if (sh + w > 64) words[wi + 1] |= v >> (64 - sh);
}

static uint64_t pack_get(const uint64_t* words, uint64_t j, int w) {
  uint64_t off = j * (uint64_t)w;
  uint64_t wi = off >> 6;
  int sh = (int)(off & 63);
  uint64_t v = words[wi] >> sh;
  if (sh + w > 64) v |= words[wi + 1] << (64 - sh);
  if (w < 64) v &= (1ull << w) - 1;
  return v;
}

/* fills ent[0..4095] with the positions of the args of superblock sb (whose
 * first arg is at position s and last at e); returns how many there are */
static uint64_t sb_positions(const or_select* h, const uint64_t* data, uint64_t s, uint64_t e,
                             uint64_t* ent) {
  uint64_t c = 0;
  for (uint64_t wi = s >> 6; wi <= (e >> 6); wi++) {
    uint64_t w = arg_word(data, h->size, wi, h->t_b);
    if (wi == (s >> 6)) w &= ~0ull << (s & 63);
    if (wi == (e >> 6) && (e & 63) != 63) w &= (1ull << ((e & 63) + 1)) - 1;
    while (w && c < 4096) { ent[c++] = (wi << 6) + __builtin_ctzll(w); w &= w - 1; }
  }
  return c;
}

/* Long/mini decision and fill for one superblock:
 * init_fast, select_support_mcl_par.hpp:525-543 (long: :528-538 via
 * init_longblock_serial :401-438; mini: :539-542 via init_miniblock_serial
 * :440-481).  Fills ent (4096 long entries or 64 mini entries, unused
 * trailing entries zero) and returns the descriptor without the offset. */
static uint64_t sb_fill(const or_select* h, const uint64_t* data, uint64_t s, uint64_t e,
                        uint64_t* ent) {
  uint64_t pos[4096];
  uint64_t c = sb_positions(h, data, s, e, pos);
  if (e - s > h->logn4) {
    int w = or_hi(e) + 1;
    memset(ent, 0, 4096 * 8);
    for (uint64_t j = 0; j < c; j++) ent[j] = pos[j];
    return (1ull << 7) | (uint64_t)w;
  }
  int w = or_hi(e - s) + 1;
  memset(ent, 0, 64 * 8);
  for (uint64_t j = 0; j < c; j += 64) ent[j / 64] = pos[j] - s;
  return (uint64_t)w;
}

static void finish_pack(or_select* h, uint64_t* ends, const uint64_t* data) {
  uint64_t nsb = h->nsb;
  h->desc = (uint64_t*)calloc(nsb ? nsb : 1, 8);
  uint64_t* ent_store = (uint64_t*)malloc((nsb ? nsb : 1) * 8);
  uint64_t total = 0;
  /* widths and kinds */
  h->has_long = 0;
  for (uint64_t i = 0; i < nsb; i++) {
    uint64_t s = h->sb_start[i], e = ends[i];
    int lng = (e - s) > h->logn4;
    int w = lng ? or_hi(e) + 1 : or_hi(e - s) + 1;
    h->desc[i] = (total << 8) | ((uint64_t)lng << 7) | (uint64_t)w;
    ent_store[i] = lng ? 64ull * w : (uint64_t)w;
    total += ent_store[i];
    if (lng) h->has_long = 1;
  }
  h->pool_nwords = total;
  h->pool = (uint64_t*)calloc(total + 1, 8);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t ii = 0; ii < (int64_t)nsb; ii++) {
    uint64_t i = (uint64_t)ii;
    uint64_t* ent = (uint64_t*)malloc(4096 * 8);
    uint64_t d = sb_fill(h, data, h->sb_start[i], ends[i], ent);
    int w = (int)(d & 127);
    int lng = (int)((d >> 7) & 1);
    uint64_t off = h->desc[i] >> 8;
    uint64_t cnt = lng ? 4096 : 64;
    for (uint64_t j = 0; j < cnt; j++) pack_put(h->pool + off, j, w, ent[j]);
    free(ent);
  }
  free(ent_store);
  /* m_superblock = int_vector<0>(sb, 0, m_logn) (select_support_mcl_par.hpp:546-549) */
  h->sb_nwords = (nsb * h->logn + 63) / 64;
  h->sb_words = (uint64_t*)calloc(h->sb_nwords + 1, 8);
  for (uint64_t i = 0; i < nsb; i++) pack_put(h->sb_words, i, (int)h->logn, h->sb_start[i]);
}

/* initData (select_support_mcl_par.hpp:619-636) */
static void init_data(or_select* h) {
  uint64_t cap = (h->size + 63) / 64 * 64;
  h->logn = (uint32_t)(or_hi(cap) + 1);
  h->logn2 = h->logn * h->logn;
  h->logn4 = h->logn2 * h->logn2;
}

/* init_slow (select_support_mcl_par.hpp:227-276): one serial sweep that
 * closes a superblock every 4096 args and at the last arg. */
static void init_slow(or_select* h, const uint64_t* data) {
  uint64_t m = 0;
  for (uint64_t i = 0; i < h->size; i++) m += ((data[i >> 6] >> (i & 63)) & 1) == (uint64_t)h->t_b;
  h->arg_cnt = m;
  if (m == 0) return;
  h->nsb = (m + 4095) / 4096;
  h->sb_start = (uint64_t*)calloc(h->nsb, 8);
  uint64_t* ends = (uint64_t*)calloc(h->nsb, 8);
  uint64_t cnt = 0, sb = 0, first = 0;
  for (uint64_t i = 0; i < h->size; i++) {
    if ((((data[i >> 6] >> (i & 63)) & 1)) != (uint64_t)h->t_b) continue;
    if (cnt % 4096 == 0) first = i;
    cnt++;
    if (cnt % 4096 == 0 || cnt == m) {
      h->sb_start[sb] = first; /* arg_position[0] */
      ends[sb] = i;            /* arg_position[(arg_cnt-1)%4096] */
      sb++;
    }
  }
  finish_pack(h, ends, data);
  free(ends);
}

/* init_fast (select_support_mcl_par.hpp:483-561): per 8192-bit chunk arg
 * counts (sum_args_serial :277-304), exclusive scan (:498), superblock
 * start/end positions found chunk by chunk (init_superblock_serial
 * :307-399), then the per-superblock long/mini fill (:525-543). */
static void init_fast(or_select* h, const uint64_t* data) {
  const uint64_t CH = 8192; /* _SCAN_BSIZE << 3 */
  uint64_t size = h->size;
  uint64_t nch = size ? 1 + (size - 1) / CH : 1;
  uint64_t* bsum = (uint64_t*)calloc(nch + 1, 8);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < (int64_t)nch; c++) {
    uint64_t s = (uint64_t)c * CH, e = s + CH < size ? s + CH : size;
    uint64_t r = 0;
    for (uint64_t wi = s >> 6; (wi << 6) < e; wi++) r += popc(arg_word(data, size, wi, h->t_b));
    bsum[c] = r;
  }
  uint64_t run = 0;
  for (uint64_t c = 0; c < nch; c++) { uint64_t t = bsum[c]; bsum[c] = run; run += t; }
  h->arg_cnt = run;
  uint64_t m = run;
  if (m == 0) { free(bsum); return; }
  h->nsb = (m + 4095) / 4096;
  h->sb_start = (uint64_t*)calloc(h->nsb, 8);
  uint64_t* ends = (uint64_t*)calloc(h->nsb, 8);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < (int64_t)nch; c++) {
    uint64_t s = (uint64_t)c * CH, e = s + CH < size ? s + CH : size;
    uint64_t k = bsum[c];
    for (uint64_t wi = s >> 6; (wi << 6) < e; wi++) {
      uint64_t w = arg_word(data, size, wi, h->t_b);
      uint64_t cw = popc(w);
      if (!cw) continue;
      /* superblock start: arg index 4096*q inside [k, k+cw) */
      uint64_t q0 = (k + 4095) / 4096 * 4096;
      if (q0 < k + cw) h->sb_start[q0 / 4096] = (wi << 6) + sel64(w, q0 - k + 1);
      /* superblock end: arg index 4096*q+4095 inside [k, k+cw) */
      uint64_t q1 = (k + 1 + 4095) / 4096 * 4096 - 1;
      if (q1 < k + cw) ends[q1 / 4096] = (wi << 6) + sel64(w, q1 - k + 1);
      /* last arg closes the last superblock */
      if (m - 1 >= k && m - 1 < k + cw) ends[h->nsb - 1] = (wi << 6) + sel64(w, m - 1 - k + 1);
      k += cw;
    }
  }
  free(bsum);
  finish_pack(h, ends, data);
  free(ends);
}

or_select* or_select_new(const uint64_t* data, uint64_t size, int t_b, int use_rule) {
  or_select* h = (or_select*)calloc(1, sizeof(or_select));
  h->size = size;
  h->t_b = t_b ? 1 : 0;
  init_data(h);
  int slow = use_rule == 1 || (use_rule == 0 && size < 100000); /* :123 */
  if (slow) init_slow(h, data); else init_fast(h, data);
  if (!h->desc) { h->desc = (uint64_t*)calloc(1, 8); }
  if (!h->sb_words) { h->sb_words = (uint64_t*)calloc(1, 8); h->sb_nwords = 0; }
  if (!h->pool) { h->pool = (uint64_t*)calloc(1, 8); h->pool_nwords = 0; }
  return h;
}

void or_select_info(const or_select* h, uint64_t info[8]) {
  info[0] = h->size; info[1] = h->arg_cnt; info[2] = h->logn; info[3] = h->logn4;
  info[4] = h->nsb; info[5] = (uint64_t)h->has_long; info[6] = h->sb_nwords; info[7] = h->pool_nwords;
}

void or_select_copy(const or_select* h, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  if (sb_words && h->sb_nwords) memcpy(sb_words, h->sb_words, h->sb_nwords * 8);
  if (desc && h->nsb) memcpy(desc, h->desc, h->nsb * 8);
  if (pool && h->pool_nwords) memcpy(pool, h->pool, h->pool_nwords * 8);
}

void or_select_free(or_select* h) {
  if (!h) return;
  free(h->sb_start); free(h->desc); free(h->sb_words); free(h->pool);
  free(h);
}

/* select_support_mcl_par.hpp:564-611, on the packed layout */
uint64_t or_select_query(const or_select* h, const uint64_t* data, uint64_t i) {
  i = i - 1;
  uint64_t sb = i >> 12, off = i & 0xFFF;
  uint64_t d = h->desc[sb];
  int w = (int)(d & 127);
  const uint64_t* blk = h->pool + (d >> 8);
  if (h->has_long && ((d >> 7) & 1)) return pack_get(blk, off, w);
  uint64_t base = pack_get(h->sb_words, sb, (int)h->logn);
  uint64_t mini = pack_get(blk, off >> 6, w);
  if ((off & 0x3F) == 0) return base + mini;
  i = i - (sb << 12) - ((off >> 6) << 6);
  uint64_t pos = base + mini + 1;
  uint64_t word_pos = pos >> 6, word_off = pos & 0x3F;
  uint64_t wd = data[word_pos];
  if (!h->t_b) wd = ~wd;
  uint64_t first = wd & (~0ull << word_off);
  uint64_t args = popc(first);
  if (args >= i) return (word_pos << 6) + sel64(first, i);
  word_pos += 1;
  uint64_t sum = args;
  wd = data[word_pos]; if (!h->t_b) wd = ~wd;
  args = popc(wd);
  while (sum + args < i) {
    sum += args;
    word_pos += 1;
    wd = data[word_pos]; if (!h->t_b) wd = ~wd;
    args = popc(wd);
  }
  return (word_pos << 6) + sel64(wd, i - sum);
}

void or_select_batch(const or_select* h, const uint64_t* data, const uint64_t* q, uint64_t nq,
                     uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nq; k++) out[k] = or_select_query(h, data, q[k]);
}

/* ------------------------------------------------------ wt_int queries */

static inline int tree_bit(const uint64_t* t, uint64_t p) { return (int)((t[p >> 6] >> (p & 63)) & 1); }

/* wt_int::operator[] (wt_int_par.hpp:519-541) */
uint64_t or_wt_access(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, uint64_t i) {
  uint64_t offset = 0, res = 0, node_size = n;
  for (int k = 0; k < L; k++) {
    res <<= 1;
    uint64_t o = or_rank1(rt, tree, offset);
    uint64_t oi = or_rank1(rt, tree, offset + i) - o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    if (tree_bit(tree, offset + i)) {
      offset += node_size - oe; node_size = oe; i = oi; res |= 1;
    } else {
      node_size = node_size - oe; i = i - oi;
    }
    offset += n;
  }
  return res;
}

/* wt_int::rank (wt_int_par.hpp:553-577) */
uint64_t or_wt_rank(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, uint64_t i,
                    uint64_t c) {
  if (L < 64 && (1ull << L) <= c) return 0;
  uint64_t offset = 0, mask = 1ull << (L - 1), node_size = n;
  for (int k = 0; k < L && i; k++) {
    uint64_t o = or_rank1(rt, tree, offset);
    uint64_t oi = or_rank1(rt, tree, offset + i) - o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    if (c & mask) { offset += node_size - oe; node_size = oe; i = oi; }
    else { node_size = node_size - oe; i = i - oi; }
    offset += n;
    mask >>= 1;
  }
  return i;
}

/* wt_int::inverse_select (wt_int_par.hpp:588-611) */
uint64_t or_wt_inverse_select(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L,
                              uint64_t i, uint64_t* c_out) {
  uint64_t c = 0, node_size = n, offset = 0;
  for (int k = 0; k < L; k++) {
    uint64_t o = or_rank1(rt, tree, offset);
    uint64_t oi = or_rank1(rt, tree, offset + i) - o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    c <<= 1;
    if (tree_bit(tree, offset + i)) { offset += node_size - oe; node_size = oe; i = oi; c |= 1; }
    else { node_size = node_size - oe; i = i - oi; }
    offset += n;
  }
  if (c_out) *c_out = c;
  return i;
}

/* wt_int::select (wt_int_par.hpp:622-660) */
uint64_t or_wt_select(const uint64_t* tree, const uint64_t* rt, const or_select* s1,
                      const or_select* s0, uint64_t n, int L, uint64_t i, uint64_t c) {
  uint64_t path_off[65], path_rank[65];
  uint64_t offset = 0, mask = 1ull << (L - 1), node_size = n;
  path_off[0] = path_rank[0] = 0;
  for (int k = 0; k < L && node_size; k++) {
    uint64_t o = or_rank1(rt, tree, offset);
    path_rank[k] = o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    if (c & mask) { offset += node_size - oe; node_size = oe; }
    else { node_size = node_size - oe; }
    offset += n;
    path_off[k + 1] = offset;
    mask >>= 1;
  }
  if (node_size == 0 || node_size < i) return UINT64_MAX;
  mask = 1;
  for (int k = L; k > 0; k--) {
    offset = path_off[k - 1];
    uint64_t o = path_rank[k - 1];
    if (c & mask) i = or_select_query(s1, tree, o + i) - offset + 1;
    else i = or_select_query(s0, tree, offset - o + i) - offset + 1;
    mask <<= 1;
  }
  return i - 1;
}

/* wt_int::lex_count (wt_int_par.hpp:715-745): out = (rank(i, c), symbols
 * smaller than c in [i, j), symbols greater than c in [i, j)) */
void or_wt_lex_count(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, uint64_t i, uint64_t j,
                     uint64_t c, uint64_t* out) {
  if (L < 64 && (1ull << L) <= c) {
    out[0] = 0; out[1] = j - i; out[2] = 0;
    return;
  }
  uint64_t offset = 0, smaller = 0, greater = 0, mask = 1ull << (L - 1), node_size = n;
  for (int k = 0; k < L; k++) {
    uint64_t o = or_rank1(rt, tree, offset);
    uint64_t oi = or_rank1(rt, tree, offset + i) - o;
    uint64_t oj = or_rank1(rt, tree, offset + j) - o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    if (c & mask) {
      offset += node_size - oe; node_size = oe;
      smaller += j - i - oj + oi; i = oi; j = oj;
    } else {
      node_size -= oe;
      greater += oj - oi; i -= oi; j -= oj;
    }
    offset += n;
    mask >>= 1;
  }
  out[0] = i; out[1] = smaller; out[2] = greater;
}

/* wt_int::lex_smaller_count (wt_int_par.hpp:758-782): out = (rank(i, c),
 * symbols smaller than c in [0, i)) */
void or_wt_lex_smaller_count(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, uint64_t i,
                             uint64_t c, uint64_t* out) {
  if (L < 64 && (1ull << L) <= c) {
    out[0] = 0; out[1] = i;
    return;
  }
  uint64_t offset = 0, result = 0, mask = 1ull << (L - 1), node_size = n;
  for (int k = 0; k < L && i; k++) {
    uint64_t o = or_rank1(rt, tree, offset);
    uint64_t oi = or_rank1(rt, tree, offset + i) - o;
    uint64_t oe = or_rank1(rt, tree, offset + node_size) - o;
    if (c & mask) { offset += node_size - oe; node_size = oe; result += i - oi; i = oi; }
    else { node_size = node_size - oe; i -= oi; }
    offset += n;
    mask >>= 1;
  }
  out[0] = i; out[1] = result;
}

/* range_search_2d (wt_int_par.hpp:801-871): points of positions [lb, rb]
 * with values in [vlb, vrb]; leaves in increasing value order, positions
 * increasing within a leaf; each reported position is found by walking up
 * with select1/select0 from the leaf. */
typedef struct {
  const uint64_t *tree, *rt;
  const or_select *s1, *s0;
  uint64_t n;
  int L, report;
  uint64_t cap, cnt;
  uint64_t *pos, *val;
  uint64_t offsets[66], obo[66];
} r2d_ctx;

static void r2d_rec(r2d_ctx* x, uint64_t lb, uint64_t rb, uint64_t vlb, uint64_t vrb, int level, uint64_t ilb,
                    uint64_t node_size, uint64_t path) {
  if (lb > rb) return;
  if (level == x->L) {
    if (x->report) {
      for (uint64_t j = lb + 1; j <= rb + 1; ++j) {
        uint64_t i = j, c = path;
        for (int k = x->L; k > 0; --k) {
          uint64_t offset = x->offsets[k - 1], o = x->obo[k - 1];
          if (c & 1) i = or_select_query(x->s1, x->tree, o + i) - offset + 1;
          else i = or_select_query(x->s0, x->tree, offset - o + i) - offset + 1;
          c >>= 1;
        }
        uint64_t q = x->cnt + (j - lb - 1);
        if (q < x->cap) { x->pos[q] = i - 1; x->val[q] = path; }
      }
    }
    x->cnt += rb - lb + 1;
    return;
  }
  uint64_t irb = ilb + (1ull << (x->L - level));
  uint64_t mid = (irb + ilb) >> 1;
  uint64_t offset = x->offsets[level];
  uint64_t o = or_rank1(x->rt, x->tree, offset);
  x->obo[level] = o;
  uint64_t olb = or_rank1(x->rt, x->tree, offset + lb);
  uint64_t orb = or_rank1(x->rt, x->tree, offset + rb + 1);
  uint64_t oend = or_rank1(x->rt, x->tree, offset + node_size);
  uint64_t zo = offset - o, zlb = offset + lb - olb, zrb = offset + rb + 1 - orb, zend = offset + node_size - oend;
  if (vlb < mid && mid) {
    uint64_t nlb = zlb - zo, nrb = zrb - zo;
    x->offsets[level + 1] = offset + x->n;
    if (nrb) r2d_rec(x, nlb, nrb - 1, vlb, vrb < mid - 1 ? vrb : mid - 1, level + 1, ilb, zend - zo, path << 1);
  }
  if (vrb >= mid) {
    uint64_t nlb = olb - o, nrb = orb - o;
    x->offsets[level + 1] = offset + x->n + (zend - zo);
    if (nrb) r2d_rec(x, nlb, nrb - 1, mid > vlb ? mid : vlb, vrb, level + 1, mid, oend - o, (path << 1) + 1);
  }
}

uint64_t or_wt_range_search_2d(const uint64_t* tree, const uint64_t* rt, const or_select* s1,
                               const or_select* s0, uint64_t n, int L, uint64_t lb, uint64_t rb, uint64_t vlb,
                               uint64_t vrb, int report, uint64_t cap, uint64_t* pos, uint64_t* val) {
  r2d_ctx x;
  memset(&x, 0, sizeof(x));
  x.tree = tree; x.rt = rt; x.s1 = s1; x.s0 = s0; x.n = n; x.L = L; x.report = report;
  x.cap = cap; x.pos = pos; x.val = val;
  if (L < 64 && vrb > (1ull << L)) vrb = 1ull << L;
  if (vlb > vrb) return 0;
  r2d_rec(&x, lb, rb, vlb, vrb, 0, 0, n, 0);
  return x.cnt;
}

/* interval_symbols (wt_int_par.hpp:684-702, recursion :119-158): the k
 * distinct symbols of [i, j) in increasing order with rank(i, c), rank(j, c) */
typedef struct {
  const uint64_t *tree, *rt;
  uint64_t n;
  int L;
  uint64_t k, cap;
  uint64_t *cs, *ri, *rj;
} isym_ctx;

static void isym_rec(isym_ctx* x, uint64_t i, uint64_t j, int level, uint64_t path, uint64_t node_size,
                     uint64_t offset) {
  if (level >= x->L) {
    if (x->k < x->cap) { x->ri[x->k] = i; x->rj[x->k] = j; x->cs[x->k] = path; }
    x->k++;
    return;
  }
  uint64_t o = or_rank1(x->rt, x->tree, offset);
  uint64_t oi = or_rank1(x->rt, x->tree, offset + i) - o;
  uint64_t oj = or_rank1(x->rt, x->tree, offset + j) - o;
  uint64_t oe = or_rank1(x->rt, x->tree, offset + node_size) - o;
  if ((j - i) - (oj - oi) > 0)
    isym_rec(x, i - oi, j - oj, level + 1, path << 1, node_size - oe, offset + x->n);
  if (oj - oi > 0)
    isym_rec(x, oi, oj, level + 1, (path << 1) | 1, oe, offset + (node_size - oe) + x->n);
}

uint64_t or_wt_interval_symbols(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, uint64_t i,
                                uint64_t j, uint64_t cap, uint64_t* cs, uint64_t* ri, uint64_t* rj) {
  if (i == j) return 0;
  if (i + 1 == j) {
    uint64_t c = 0, r = or_wt_inverse_select(tree, rt, n, L, i, &c);
    if (cap) { cs[0] = c; ri[0] = r; rj[0] = r + 1; }
    return 1;
  }
  isym_ctx x = {tree, rt, n, L, 0, cap, cs, ri, rj};
  isym_rec(&x, i, j, 0, 0, n, 0);
  return x.k;
}

/* expand(v) (wt_int_par.hpp:966-984); nodes are (offset, size, level, sym) */
void or_wt_expand(const uint64_t* tree, const uint64_t* rt, uint64_t n, const uint64_t* v, uint64_t* left,
                  uint64_t* right) {
  uint64_t offset_rank = or_rank1(rt, tree, v[0]);
  uint64_t ones = or_rank1(rt, tree, v[0] + v[1]) - offset_rank;
  left[0] = v[0] + n; left[1] = v[1] - ones; left[2] = v[2] + 1; left[3] = v[3] << 1;
  right[0] = v[0] + n + left[1]; right[1] = ones; right[2] = v[2] + 1; right[3] = (v[3] << 1) | 1;
}

/* expand(v, ranges) (wt_int_par.hpp:1027-1048): closed ranges [s, e] of v
 * mapped to its children, in unsigned 64-bit arithmetic */
void or_wt_expand_ranges(const uint64_t* tree, const uint64_t* rt, const uint64_t* v, const uint64_t* ranges,
                         uint64_t nr, uint64_t* left, uint64_t* right) {
  uint64_t v_sp_rank = or_rank1(rt, tree, v[0]);
  for (uint64_t q = 0; q < nr; q++) {
    uint64_t s = ranges[2 * q], e = ranges[2 * q + 1];
    uint64_t sp_rank = or_rank1(rt, tree, v[0] + s);
    uint64_t right_size = or_rank1(rt, tree, v[0] + e + 1) - sp_rank;
    uint64_t left_size = (e - s + 1) - right_size;
    uint64_t right_sp = sp_rank - v_sp_rank, left_sp = s - right_sp;
    left[2 * q] = left_sp; left[2 * q + 1] = left_sp + left_size - 1;
    right[2 * q] = right_sp; right[2 * q + 1] = right_sp + right_size - 1;
  }
}

void or_wt_lex_count_batch(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, const uint64_t* i,
                           const uint64_t* j, const uint64_t* c, uint64_t nq, uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nq; k++) or_wt_lex_count(tree, rt, n, L, i[k], j[k], c[k], out + 3 * k);
}

void or_wt_lex_smaller_count_batch(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L,
                                   const uint64_t* i, const uint64_t* c, uint64_t nq, uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nq; k++) or_wt_lex_smaller_count(tree, rt, n, L, i[k], c[k], out + 2 * k);
}

void or_wt_range_count_batch(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, const uint64_t* lb,
                             const uint64_t* rb, const uint64_t* vlb, const uint64_t* vrb, uint64_t nq,
                             uint64_t* out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < (int64_t)nq; k++)
    out[k] = or_wt_range_search_2d(tree, rt, NULL, NULL, n, L, lb[k], rb[k], vlb[k], vrb[k], 0, 0, NULL, NULL);
}

void or_wt_access_batch(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L,
                        const uint64_t* idx, uint64_t nq, uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nq; k++) out[k] = or_wt_access(tree, rt, n, L, idx[k]);
}

void or_wt_rank_batch(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L,
                      const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nq; k++) out[k] = or_wt_rank(tree, rt, n, L, idx[k], sym[k]);
}

/* ------------------------------------------------------------ FM-index core */

int or_suffix_array_u8(const uint8_t* s, int64_t n, int64_t* sa) {
  if (n <= 0) return 0;
  int64_t m = n > 256 ? n : 256;
  int64_t* x = (int64_t*)malloc(sizeof(int64_t) * n);
  int64_t* y = (int64_t*)malloc(sizeof(int64_t) * n);
  int64_t* c = (int64_t*)malloc(sizeof(int64_t) * (m + 1));
  if (!x || !y || !c) {
    free(x); free(y); free(c);
    return -1;
  }
  int64_t classes = 256;
  memset(c, 0, sizeof(int64_t) * (m + 1));
  for (int64_t i = 0; i < n; i++) c[x[i] = s[i]]++;
  for (int64_t i = 1; i < classes; i++) c[i] += c[i - 1];
  for (int64_t i = n - 1; i >= 0; i--) sa[--c[x[i]]] = i;
  for (int64_t k = 1; k < n; k <<= 1) {
    /* order by the second key: suffixes without one first, then by sa */
    int64_t p = 0;
    for (int64_t i = n - k; i < n; i++) y[p++] = i;
    for (int64_t i = 0; i < n; i++)
      if (sa[i] >= k) y[p++] = sa[i] - k;
    /* stable counting sort by the first key */
    memset(c, 0, sizeof(int64_t) * (classes + 1));
    for (int64_t i = 0; i < n; i++) c[x[y[i]]]++;
    for (int64_t i = 1; i < classes; i++) c[i] += c[i - 1];
    for (int64_t i = n - 1; i >= 0; i--) sa[--c[x[y[i]]]] = y[i];
    /* new classes of the first 2k bytes */
    int64_t* t = x; x = y; y = t;
    p = 1;
    x[sa[0]] = 0;
    for (int64_t i = 1; i < n; i++) {
      const int64_t a = sa[i - 1], b = sa[i];
      const int64_t a2 = a + k < n ? y[a + k] : -1, b2 = b + k < n ? y[b + k] : -1;
      x[b] = (y[a] == y[b] && a2 == b2) ? p - 1 : p++;
    }
    if (p >= n) break;
    classes = p;
  }
  free(x); free(y); free(c);
  return 0;
}

void or_bwt_u8(const uint8_t* s, const int64_t* sa, int64_t n, uint8_t* bwt) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) bwt[i] = s[sa[i] ? sa[i] - 1 : n - 1];
}

void or_fm_count(const uint64_t* tree, const uint64_t* rt, uint64_t n, int L, const uint64_t* C,
                 uint64_t sigma, const uint8_t* pat, const uint64_t* off, uint64_t npat, uint64_t* out) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t p = 0; p < (int64_t)npat; p++) {
    uint64_t sp = 0, ep = n;
    for (uint64_t i = off[p + 1]; i > off[p] && sp < ep; i--) {
      const uint64_t c = pat[i - 1];
      if (c >= sigma) {
        ep = sp;
        break;
      }
      sp = C[c] + or_wt_rank(tree, rt, n, L, sp, c);
      ep = C[c] + or_wt_rank(tree, rt, n, L, ep, c);
    }
    out[p] = ep > sp ? ep - sp : 0;
  }
}
