// wtg_capi.cu -- the extern "C" boundary (include/wtg.h): handles, argument
// checks, host<->device copies and error reporting around the kernels.
#include <cstring>
#include <new>
#include <string>

#include "wtg_tree.cuh"

struct wtg_tree {
  wtg::TreeImpl t;
};

struct wtg_batch {
  wtg::BatchImpl* b = nullptr;
};

struct wtg_lsel {
  wtg::LselImpl* m = nullptr;
  wtg::DevBuf qbuf;
};

struct wtg_huff {
  wtg::HuffImpl* h = nullptr;
};

struct wtg_bv {
  wtg::BvSupport bv;
  wtg::DevBuf words;  // device copy for host-input builds
  wtg::DevBuf err;
  wtg::DevBuf qbuf;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
};

using namespace wtg;

namespace {

constexpr int MAX_LEVELS = 24;
// inputs of at least this many symbols are copied in pieces by wtg_tree_build_out
constexpr uint64_t IN_PIECE_MIN_SYMBOLS = 1ull << 22;

int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(WTG_ERR_CUDA, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
  return WTG_OK;
}

int check_seq_args(uint64_t n, int eb, int levels, uint32_t flags) {
  if (eb != 1 && eb != 2 && eb != 4 && eb != 8) return fail(WTG_ERR_INVALID, "elem_bytes must be 1, 2, 4 or 8");
  if (levels < 0 || levels > MAX_LEVELS) return fail(WTG_ERR_INVALID, "levels must be 0 (derive) or 1..24");
  if (n >= (1ull << 32)) return fail(WTG_ERR_INVALID, "n must be below 2^32");
  if (flags & ~WTG_ALL) return fail(WTG_ERR_INVALID, "unknown flags");
  return WTG_OK;
}

int sync_and_check(cudaStream_t s, const uint32_t* d_err) {
  WTG_CK(cudaStreamSynchronize(s));
  uint32_t e = 0;
  if (d_err) {
    WTG_CK(cudaMemcpy(&e, d_err, sizeof(e), cudaMemcpyDeviceToHost));
  }
  if (e == DERR_LOOKBACK_TIMEOUT) return fail(WTG_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  if (e == DERR_BAD_INDEX) return fail(WTG_ERR_CUDA, "a computed index fell outside its buffer (inconsistent tables)");
  if (e) return fail(WTG_ERR_CUDA, "device reported error code " + std::to_string(e));
  return WTG_OK;
}

uint64_t rank_words_of(uint64_t size) {
  if (size == 0) return 2;
  uint64_t cap = (size + 63) / 64 * 64;
  return ((cap >> 9) + 1) << 1;
}

int build_tree_common(wtg_tree* T, const void* d_seq, uint64_t n, int eb, int levels, uint32_t flags) {
  TreeImpl& t = T->t;
  int rc;
  if (levels == 0) {
    if ((rc = tree_levels_from_max(t, d_seq, n, eb, &levels))) return rc;
    if (levels > MAX_LEVELS) return fail(WTG_ERR_RANGE, "derived levels exceed 24");
  }
  return tree_build(t, d_seq, n, eb, levels, flags);
}

// runs `launch` on device copies of host query arrays
template <typename F>
int host_query(DevBuf& qbuf, cudaStream_t s, const uint64_t* const* ins, int nin, uint64_t nq,
               uint64_t* const* outs, int nout, const uint32_t* d_err, F launch) {
  int rc;
  if (nq == 0) return WTG_OK;
  if ((rc = qbuf.ensure((size_t)(nin + nout) * nq * sizeof(uint64_t), s))) return rc;
  uint64_t* d = qbuf.as<uint64_t>();
  for (int k = 0; k < nin; ++k)
    WTG_CK(cudaMemcpyAsync(d + k * nq, ins[k], nq * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  const uint64_t* din[4];
  uint64_t* dout[4];
  for (int k = 0; k < nin; ++k) din[k] = d + k * nq;
  for (int k = 0; k < nout; ++k) dout[k] = d + (nin + k) * nq;
  if ((rc = launch(din, dout))) return rc;
  for (int k = 0; k < nout; ++k)
    WTG_CK(cudaMemcpyAsync(outs[k], dout[k], nq * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, d_err);
}

// Variable-size answers: the query arrays go to the device, `count` fills
// the per-query counts; when `fill` is given (nv output arrays, cap > 0)
// the counts are scanned into offsets, `fill` writes up to cap answers, and
// the first min(total, cap) of each output array come back.
template <typename C, typename F>
int host_variable_query(TreeImpl& t, const uint64_t* const* ins, int nin, uint64_t nq, uint64_t* counts_out,
                        uint64_t cap, uint64_t* const* outs, int nv, C count, F fill) {
  int rc;
  cudaStream_t s = t.stream;
  if (nq == 0) return WTG_OK;
  if ((rc = t.qbuf.ensure((size_t)(nin * nq + nq + nq + 1) * sizeof(uint64_t), s))) return rc;
  uint64_t* d = t.qbuf.as<uint64_t>();
  const uint64_t* din[4];
  for (int k = 0; k < nin; ++k) {
    WTG_CK(cudaMemcpyAsync(d + k * nq, ins[k], nq * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    din[k] = d + k * nq;
  }
  uint64_t* d_cnt = d + nin * nq;
  uint64_t* d_off = d_cnt + nq;
  if ((rc = count(din, d_cnt))) return rc;
  WTG_CK(cudaMemcpyAsync(counts_out, d_cnt, nq * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (!nv || !cap) return sync_and_check(s, t.err.as<uint32_t>());
  if ((rc = answer_offsets(d_cnt, nq, d_off, t.scan_tmp, t.err.as<uint32_t>(), s))) return rc;
  uint64_t total = 0;
  WTG_CK(cudaMemcpyAsync(&total, d_off + nq, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if ((rc = sync_and_check(s, t.err.as<uint32_t>()))) return rc;
  const uint64_t m = std::min(total, cap);
  if (!m) return WTG_OK;
  if ((rc = t.qout.ensure((size_t)nv * m * sizeof(uint64_t), s))) return rc;
  uint64_t* dout[4];
  for (int k = 0; k < nv; ++k) dout[k] = t.qout.as<uint64_t>() + k * m;
  if ((rc = fill(din, (const uint64_t*)d_off, m, dout))) return rc;
  for (int k = 0; k < nv; ++k)
    WTG_CK(cudaMemcpyAsync(outs[k], dout[k], m * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, t.err.as<uint32_t>());
}

void fill_select_info(const BvSupport& bv, int t_b, uint64_t info[8]) {
  const SelectDev& sd = bv.sel[t_b];
  info[0] = bv.size;
  info[1] = sd.arg_cnt;
  info[2] = sd.logn;
  info[3] = sd.logn4;
  info[4] = sd.nsb;
  info[5] = sd.has_long;
  info[6] = sd.sb_nwords;
  info[7] = sd.pool_nwords;
}

int copy_select(const BvSupport& bv, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool, cudaStream_t s) {
  if (!(bv.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select support not built");
  const SelectDev& sd = bv.sel[t_b];
  if (sd.sb_nwords && sb_words)
    WTG_CK(cudaMemcpyAsync(sb_words, sd.sb_words.p, sd.sb_nwords * 8, cudaMemcpyDeviceToHost, s));
  if (sd.nsb && desc) WTG_CK(cudaMemcpyAsync(desc, sd.desc.p, sd.nsb * 8, cudaMemcpyDeviceToHost, s));
  if (sd.pool_nwords && pool) WTG_CK(cudaMemcpyAsync(pool, sd.pool.p, sd.pool_nwords * 8, cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaStreamSynchronize(s));
  return WTG_OK;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ trees

int wtg_tree_build(const void* seq, uint64_t n, int elem_bytes, int levels, uint32_t flags, wtg_tree** out) {
  int rc;
  if (!out || (!seq && n)) return fail(WTG_ERR_INVALID, "null argument");
  if ((rc = check_seq_args(n, elem_bytes, levels, flags))) return rc;
  if ((rc = check_device())) return rc;
  wtg_tree* T = *out;
  const bool fresh = (T == nullptr);
  if (fresh) {
    T = new (std::nothrow) wtg_tree();
    if (!T) return fail(WTG_ERR_OOM, "host allocation failed");
  }
  TreeImpl& t = T->t;
  if (!t.own_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      if (fresh) delete T;
      return cuda_fail(e, "cudaStreamCreate");
    }
    t.own_stream = true;
  }
  if ((rc = t.seq.ensure(n * elem_bytes, t.stream)) == WTG_OK) {
    cudaError_t ce = cudaSuccess;
    if (n) ce = cudaMemcpyAsync(t.seq.p, seq, n * elem_bytes, cudaMemcpyHostToDevice, t.stream);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaMemcpyAsync(seq)");
  }
  if (rc == WTG_OK) rc = build_tree_common(T, t.seq.p, n, elem_bytes, levels, flags);
  if (rc == WTG_OK) rc = sync_and_check(t.stream, t.err.as<uint32_t>());
  if (rc != WTG_OK) {
    if (fresh) wtg_tree_free(T);
    return rc;
  }
  *out = T;
  return WTG_OK;
}

int wtg_tree_build_out(const void* seq, uint64_t n, int elem_bytes, int levels, uint32_t flags, uint64_t* bits_dst,
                       uint64_t* rank_dst, wtg_tree** out) {
  int rc;
  if (!out || (!seq && n)) return fail(WTG_ERR_INVALID, "null argument");
  if ((rc = check_seq_args(n, elem_bytes, levels, flags))) return rc;
  if (levels == 0 && (bits_dst || rank_dst))
    return fail(WTG_ERR_INVALID, "give the levels explicitly when outputs are copied during the build");
  if (rank_dst && !(flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "rank_dst needs WTG_RANK");
  if ((rc = check_device())) return rc;
  wtg_tree* T = *out;
  const bool fresh = (T == nullptr);
  if (fresh) {
    T = new (std::nothrow) wtg_tree();
    if (!T) return fail(WTG_ERR_OOM, "host allocation failed");
  }
  TreeImpl& t = T->t;
  cudaError_t e = cudaSuccess;
  if (!t.own_stream) {
    e = cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) t.own_stream = true;
  }
  if (e == cudaSuccess && !t.copy_stream) e = cudaStreamCreateWithFlags(&t.copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !t.copy_ev) e = cudaEventCreateWithFlags(&t.copy_ev, cudaEventDisableTiming);
  if (e == cudaSuccess && !t.rank_ev) e = cudaEventCreateWithFlags(&t.rank_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (fresh) wtg_tree_free(T);
    return cuda_fail(e, "stream/event create");
  }
  // a large page-locked input is copied in pieces on in_stream, and the
  // build's pre-pass counts each piece as it lands (the levels are known, so
  // nothing else reads the input before the pre-pass is done)
  const int pieces = (levels > 0 && n >= IN_PIECE_MIN_SYMBOLS && host_page_locked(seq)) ? TreeImpl::IN_PIECES_MAX : 0;
  if (e == cudaSuccess && pieces && !t.in_stream) e = cudaStreamCreateWithFlags(&t.in_stream, cudaStreamNonBlocking);
  for (int i = 0; e == cudaSuccess && i < pieces; ++i)
    if (!t.in_ev[i]) e = cudaEventCreateWithFlags(&t.in_ev[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (fresh) wtg_tree_free(T);
    return cuda_fail(e, "stream/event create");
  }
  if ((rc = t.seq.ensure(n * elem_bytes, t.stream)) == WTG_OK) {
    cudaError_t ce = cudaSuccess;
    if (pieces) {
      // the pieces start after everything queued on the build stream (the
      // buffer's allocation, a previous build's reads of it)
      const uint64_t nchunks = (n + 511) / 512;
      const uint64_t per = (nchunks + pieces - 1) / pieces;
      ce = cudaEventRecord(t.in_ev[0], t.stream);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(t.in_stream, t.in_ev[0], 0);
      for (int i = 0; ce == cudaSuccess && i < pieces; ++i) {
        const uint64_t lo = std::min<uint64_t>(n, (uint64_t)i * per * 512);
        const uint64_t hi = std::min<uint64_t>(n, ((uint64_t)i + 1) * per * 512);
        if (hi > lo)
          ce = cudaMemcpyAsync((char*)t.seq.p + lo * elem_bytes, (const char*)seq + lo * elem_bytes,
                               (hi - lo) * elem_bytes, cudaMemcpyHostToDevice, t.in_stream);
        if (ce == cudaSuccess) ce = cudaEventRecord(t.in_ev[i], t.in_stream);
      }
      t.in_pieces = pieces;
      t.in_piece_chunks = per;
    } else if (n) {
      ce = cudaMemcpyAsync(t.seq.p, seq, n * elem_bytes, cudaMemcpyHostToDevice, t.stream);
    }
    if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaMemcpyAsync(seq)");
  }
  t.host_bits = bits_dst;
  t.host_rank = rank_dst;
  if (rc == WTG_OK) rc = build_tree_common(T, t.seq.p, n, elem_bytes, levels, flags);
  t.host_bits = nullptr;
  t.host_rank = nullptr;
  t.in_pieces = 0;
  if (rc == WTG_OK) rc = sync_and_check(t.stream, t.err.as<uint32_t>());
  if (rc == WTG_OK) {
    const cudaError_t ce = cudaStreamSynchronize(t.copy_stream);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "copies of the outputs");
  }
  if (rc != WTG_OK) {
    // a build that stopped before its pre-pass waited for every piece
    // leaves no copy in flight into the tree's input buffer
    if (pieces) cudaStreamSynchronize(t.in_stream);
    if (fresh) wtg_tree_free(T);
    return rc;
  }
  *out = T;
  return WTG_OK;
}

int wtg_tree_build_device(const void* d_seq, uint64_t n, int elem_bytes, int levels, uint32_t flags, void* stream,
                          wtg_tree** out) {
  int rc;
  if (!out || (!d_seq && n)) return fail(WTG_ERR_INVALID, "null argument");
  if ((rc = check_seq_args(n, elem_bytes, levels, flags))) return rc;
  if ((rc = check_device())) return rc;
  wtg_tree* T = *out;
  bool fresh = false;
  if (!T) {
    T = new (std::nothrow) wtg_tree();
    if (!T) return fail(WTG_ERR_OOM, "host allocation failed");
    fresh = true;
  }
  if (T->t.own_stream) {
    cudaStreamSynchronize(T->t.stream);
    cudaStreamDestroy(T->t.stream);
    T->t.own_stream = false;
  }
  T->t.stream = (cudaStream_t)stream;
  rc = build_tree_common(T, d_seq, n, elem_bytes, levels, flags);
  if (rc != WTG_OK) {
    if (fresh) wtg_tree_free(T);
    return rc;
  }
  *out = T;
  return WTG_OK;
}

int wtg_tree_sync(wtg_tree* T) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
}

int wtg_tree_free(wtg_tree* T) {
  if (!T) return WTG_OK;
  cudaStream_t s = T->t.stream;
  tree_release(T->t);
  cudaStreamSynchronize(s);
  if (T->t.own_stream) cudaStreamDestroy(s);
  delete T;
  return WTG_OK;
}

int wtg_tree_info(wtg_tree* T, uint64_t info[4]) {
  if (!T || !info) return fail(WTG_ERR_INVALID, "null argument");
  info[0] = T->t.n;
  info[1] = (uint64_t)T->t.levels;
  info[2] = T->t.bit_words;
  info[3] = (T->t.flags & WTG_RANK) ? rank_words_of(T->t.n * (uint64_t)T->t.levels) : 0;
  return WTG_OK;
}

int wtg_tree_select_info(wtg_tree* T, int t_b, uint64_t info[8]) {
  if (!T || !info || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  if (!(T->t.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select support not built");
  fill_select_info(T->t.bv, t_b, info);
  return WTG_OK;
}

int wtg_tree_get_bits(wtg_tree* T, uint64_t* dst, uint64_t nwords) {
  if (!T || (!dst && nwords)) return fail(WTG_ERR_INVALID, "null argument");
  if (nwords != T->t.bit_words) return fail(WTG_ERR_INVALID, "nwords does not match the tree");
  if (nwords) WTG_CK(cudaMemcpyAsync(dst, T->t.bits.p, nwords * 8, cudaMemcpyDeviceToHost, T->t.stream));
  return sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
}

int wtg_tree_get_nodes(wtg_tree* T, int index_bytes, uint64_t n_entries, void* dst) {
  int rc;
  if (!T || (!dst && n_entries)) return fail(WTG_ERR_INVALID, "null argument");
  if (index_bytes != 4 && index_bytes != 8) return fail(WTG_ERR_INVALID, "index_bytes must be 4 or 8");
  TreeImpl& t = T->t;
  const size_t bytes = n_entries * 5 * (size_t)index_bytes;
  if ((rc = t.nodes.ensure(bytes, t.stream))) return rc;
  if ((rc = tree_nodes(t, index_bytes, n_entries, t.nodes.p))) return rc;
  if (bytes) WTG_CK(cudaMemcpyAsync(dst, t.nodes.p, bytes, cudaMemcpyDeviceToHost, t.stream));
  return sync_and_check(t.stream, t.err.as<uint32_t>());
}

int wtg_tree_get_rank(wtg_tree* T, uint64_t* dst, uint64_t nwords) {
  if (!T || !dst) return fail(WTG_ERR_INVALID, "null argument");
  if (!(T->t.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "rank support not built");
  if (nwords != rank_words_of(T->t.n * (uint64_t)T->t.levels)) return fail(WTG_ERR_INVALID, "nwords mismatch");
  WTG_CK(cudaMemcpyAsync(dst, T->t.bv.rank.p, nwords * 8, cudaMemcpyDeviceToHost, T->t.stream));
  return sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
}

int wtg_tree_get_select(wtg_tree* T, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  if (!T || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  int rc = copy_select(T->t.bv, t_b, sb_words, desc, pool, T->t.stream);
  if (rc) return rc;
  return sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
}

int wtg_tree_device_ptrs(wtg_tree* T, uint64_t ptrs[8]) {
  if (!T || !ptrs) return fail(WTG_ERR_INVALID, "null argument");
  const BvSupport& bv = T->t.bv;
  ptrs[0] = (uint64_t)T->t.bits.p;
  ptrs[1] = (uint64_t)bv.rank.p;
  ptrs[2] = (uint64_t)bv.sel[1].sb_words.p;
  ptrs[3] = (uint64_t)bv.sel[1].desc.p;
  ptrs[4] = (uint64_t)bv.sel[1].pool.p;
  ptrs[5] = (uint64_t)bv.sel[0].sb_words.p;
  ptrs[6] = (uint64_t)bv.sel[0].desc.p;
  ptrs[7] = (uint64_t)bv.sel[0].pool.p;
  return WTG_OK;
}

// ---------------------------------------------------------------- queries

int wtg_query_access(wtg_tree* T, const uint64_t* idx, uint64_t nq, uint64_t* out) {
  if (!T || (nq && (!idx || !out))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[1] = {idx};
  uint64_t* outs[1] = {out};
  return host_query(t.qbuf, t.stream, ins, 1, nq, outs, 1, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_access(t, din[0], nq, dout[0], t.stream);
                    });
}

int wtg_query_rank(wtg_tree* T, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out) {
  if (!T || (nq && (!idx || !sym || !out))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[2] = {idx, sym};
  uint64_t* outs[1] = {out};
  return host_query(t.qbuf, t.stream, ins, 2, nq, outs, 1, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_rank(t, din[0], din[1], nq, dout[0], t.stream);
                    });
}

int wtg_query_inverse_select(wtg_tree* T, const uint64_t* idx, uint64_t nq, uint64_t* rank_out, uint64_t* sym_out) {
  if (!T || (nq && (!idx || !rank_out || !sym_out))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[1] = {idx};
  uint64_t* outs[2] = {rank_out, sym_out};
  return host_query(t.qbuf, t.stream, ins, 1, nq, outs, 2, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_inverse_select(t, din[0], nq, dout[0], dout[1], t.stream);
                    });
}

int wtg_query_select(wtg_tree* T, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out) {
  if (!T || (nq && (!i || !sym || !out))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[2] = {i, sym};
  uint64_t* outs[1] = {out};
  return host_query(t.qbuf, t.stream, ins, 2, nq, outs, 1, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_select(t, din[0], din[1], nq, dout[0], t.stream);
                    });
}

int wtg_query_access_device(wtg_tree* T, const uint64_t* d_idx, uint64_t nq, uint64_t* d_out, void* stream) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return launch_wt_access(T->t, d_idx, nq, d_out, (cudaStream_t)stream);
}

int wtg_query_rank_device(wtg_tree* T, const uint64_t* d_idx, const uint64_t* d_sym, uint64_t nq, uint64_t* d_out,
                          void* stream) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return launch_wt_rank(T->t, d_idx, d_sym, nq, d_out, (cudaStream_t)stream);
}

// ------------------------------------------------------- range queries

int wtg_query_lex_count(wtg_tree* T, const uint64_t* i, const uint64_t* j, const uint64_t* c, uint64_t nq,
                        uint64_t* rank_out, uint64_t* smaller_out, uint64_t* greater_out) {
  if (!T || (nq && (!i || !j || !c || !rank_out || !smaller_out || !greater_out)))
    return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[3] = {i, j, c};
  uint64_t* outs[3] = {rank_out, smaller_out, greater_out};
  return host_query(t.qbuf, t.stream, ins, 3, nq, outs, 3, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_lex_count(t, din[0], din[1], din[2], nq, dout[0], dout[1], dout[2],
                                                 t.stream);
                    });
}

int wtg_query_lex_smaller_count(wtg_tree* T, const uint64_t* i, const uint64_t* c, uint64_t nq, uint64_t* rank_out,
                                uint64_t* smaller_out) {
  if (!T || (nq && (!i || !c || !rank_out || !smaller_out))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[2] = {i, c};
  uint64_t* outs[2] = {rank_out, smaller_out};
  return host_query(t.qbuf, t.stream, ins, 2, nq, outs, 2, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_wt_lex_smaller_count(t, din[0], din[1], nq, dout[0], dout[1], t.stream);
                    });
}

int wtg_query_range_search_2d(wtg_tree* T, const uint64_t* lb, const uint64_t* rb, const uint64_t* vlb,
                              const uint64_t* vrb, uint64_t nq, uint64_t* count_out, uint64_t cap, uint64_t* pos_out,
                              uint64_t* val_out) {
  if (!T || (nq && (!lb || !rb || !vlb || !vrb || !count_out))) return fail(WTG_ERR_INVALID, "null argument");
  if ((pos_out == nullptr) != (val_out == nullptr)) return fail(WTG_ERR_INVALID, "pos_out and val_out go together");
  TreeImpl& t = T->t;
  const uint64_t* ins[4] = {lb, rb, vlb, vrb};
  uint64_t* outs[2] = {pos_out, val_out};
  const int nv = pos_out ? 2 : 0;
  if (nv && cap && (t.flags & WTG_ALL) != WTG_ALL)
    return fail(WTG_ERR_INVALID, "range_search_2d with report needs rank and both selects");
  return host_variable_query(
      t, ins, 4, nq, count_out, cap, outs, nv,
      [&](const uint64_t** din, uint64_t* d_cnt) {
        return launch_wt_range_count(t, din[0], din[1], din[2], din[3], nq, d_cnt, t.stream);
      },
      [&](const uint64_t** din, const uint64_t* d_off, uint64_t m, uint64_t** dout) {
        return launch_wt_range_report(t, din[0], din[1], din[2], din[3], nq, d_off, m, dout[0], dout[1], t.stream);
      });
}

int wtg_query_interval_symbols(wtg_tree* T, const uint64_t* i, const uint64_t* j, uint64_t nq, uint64_t* k_out,
                               uint64_t cap, uint64_t* cs_out, uint64_t* rank_i_out, uint64_t* rank_j_out) {
  if (!T || (nq && (!i || !j || !k_out))) return fail(WTG_ERR_INVALID, "null argument");
  const int given = (cs_out != nullptr) + (rank_i_out != nullptr) + (rank_j_out != nullptr);
  if (given != 0 && given != 3) return fail(WTG_ERR_INVALID, "cs_out, rank_i_out and rank_j_out go together");
  TreeImpl& t = T->t;
  const uint64_t* ins[2] = {i, j};
  uint64_t* outs[3] = {cs_out, rank_i_out, rank_j_out};
  return host_variable_query(
      t, ins, 2, nq, k_out, cap, outs, given,
      [&](const uint64_t** din, uint64_t* d_cnt) {
        return launch_wt_interval_symbols(t, din[0], din[1], nq, d_cnt, nullptr, 0, nullptr, nullptr, nullptr,
                                          t.stream);
      },
      [&](const uint64_t** din, const uint64_t* d_off, uint64_t m, uint64_t** dout) {
        return launch_wt_interval_symbols(t, din[0], din[1], nq, nullptr, d_off, m, dout[0], dout[1], dout[2],
                                          t.stream);
      });
}

int wtg_query_expand(wtg_tree* T, const uint64_t* nodes, uint64_t nn, uint64_t* left, uint64_t* right) {
  if (!T || (nn && (!nodes || !left || !right))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  int rc;
  if (!nn) return WTG_OK;
  cudaStream_t s = t.stream;
  if ((rc = t.qbuf.ensure((size_t)12 * nn * sizeof(uint64_t), s))) return rc;
  uint64_t* d = t.qbuf.as<uint64_t>();
  WTG_CK(cudaMemcpyAsync(d, nodes, 4 * nn * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  if ((rc = launch_wt_expand(t, d, nn, d + 4 * nn, d + 8 * nn, s))) return rc;
  WTG_CK(cudaMemcpyAsync(left, d + 4 * nn, 4 * nn * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(right, d + 8 * nn, 4 * nn * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, t.err.as<uint32_t>());
}

int wtg_query_expand_ranges(wtg_tree* T, const uint64_t v[4], const uint64_t* ranges, uint64_t nr, uint64_t* left,
                            uint64_t* right) {
  if (!T || !v || (nr && (!ranges || !left || !right))) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl& t = T->t;
  int rc;
  if (!nr) return WTG_OK;
  cudaStream_t s = t.stream;
  if ((rc = t.qbuf.ensure((size_t)6 * nr * sizeof(uint64_t), s))) return rc;
  uint64_t* d = t.qbuf.as<uint64_t>();
  WTG_CK(cudaMemcpyAsync(d, ranges, 2 * nr * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  if ((rc = launch_wt_expand_ranges(t, v[0], d, nr, d + 2 * nr, d + 4 * nr, s))) return rc;
  WTG_CK(cudaMemcpyAsync(left, d + 2 * nr, 2 * nr * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  WTG_CK(cudaMemcpyAsync(right, d + 4 * nr, 2 * nr * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, t.err.as<uint32_t>());
}

int wtg_query_lex_count_device(wtg_tree* T, const uint64_t* d_i, const uint64_t* d_j, const uint64_t* d_c,
                               uint64_t nq, uint64_t* d_rank, uint64_t* d_smaller, uint64_t* d_greater,
                               void* stream) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return launch_wt_lex_count(T->t, d_i, d_j, d_c, nq, d_rank, d_smaller, d_greater, (cudaStream_t)stream);
}

int wtg_query_range_count_device(wtg_tree* T, const uint64_t* d_lb, const uint64_t* d_rb, const uint64_t* d_vlb,
                                 const uint64_t* d_vrb, uint64_t nq, uint64_t* d_count, void* stream) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return launch_wt_range_count(T->t, d_lb, d_rb, d_vlb, d_vrb, nq, d_count, (cudaStream_t)stream);
}

// ----------------------------------------------------- standalone bitvectors

static int bv_common(wtg_bv* B, const uint64_t* d_words, uint64_t size, uint32_t flags) {
  int rc;
  if ((rc = B->err.ensure(sizeof(uint32_t), B->stream))) return rc;
  WTG_CK(cudaMemsetAsync(B->err.p, 0, sizeof(uint32_t), B->stream));
  return bv_build(B->bv, d_words, size, flags, B->err.as<uint32_t>(), B->stream);
}

int wtg_bv_build(const uint64_t* words, uint64_t size_bits, uint32_t flags, wtg_bv** out) {
  int rc;
  if (!out || (!words && size_bits)) return fail(WTG_ERR_INVALID, "null argument");
  *out = nullptr;
  if (flags & ~WTG_ALL) return fail(WTG_ERR_INVALID, "unknown flags");
  if (size_bits >= (1ull << 40)) return fail(WTG_ERR_INVALID, "bitvector too large");
  if ((rc = check_device())) return rc;
  wtg_bv* B = new (std::nothrow) wtg_bv();
  if (!B) return fail(WTG_ERR_OOM, "host allocation failed");
  cudaError_t e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete B;
    return cuda_fail(e, "cudaStreamCreate");
  }
  B->own_stream = true;
  const uint64_t W = (size_bits + 63) / 64;
  rc = B->words.ensure((W + 2) * 8, B->stream);
  if (rc == WTG_OK) {
    cudaError_t ce = cudaMemsetAsync(B->words.p, 0, (W + 2) * 8, B->stream);
    if (ce == cudaSuccess && W) ce = cudaMemcpyAsync(B->words.p, words, W * 8, cudaMemcpyHostToDevice, B->stream);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "copy bitvector");
  }
  if (rc == WTG_OK) rc = bv_common(B, B->words.as<uint64_t>(), size_bits, flags);
  if (rc == WTG_OK) rc = sync_and_check(B->stream, B->err.as<uint32_t>());
  if (rc != WTG_OK) {
    wtg_bv_free(B);
    return rc;
  }
  *out = B;
  return WTG_OK;
}

int wtg_bv_build_device(const uint64_t* d_words, uint64_t size_bits, uint32_t flags, void* stream, wtg_bv** out) {
  int rc;
  if (!out || (!d_words && size_bits)) return fail(WTG_ERR_INVALID, "null argument");
  if (flags & ~WTG_ALL) return fail(WTG_ERR_INVALID, "unknown flags");
  if (size_bits >= (1ull << 40)) return fail(WTG_ERR_INVALID, "bitvector too large");
  if ((rc = check_device())) return rc;
  wtg_bv* B = *out;
  bool fresh = false;
  if (!B) {
    B = new (std::nothrow) wtg_bv();
    if (!B) return fail(WTG_ERR_OOM, "host allocation failed");
    fresh = true;
  }
  B->stream = (cudaStream_t)stream;
  rc = bv_common(B, d_words, size_bits, flags);
  if (rc != WTG_OK) {
    if (fresh) wtg_bv_free(B);
    return rc;
  }
  *out = B;
  return WTG_OK;
}

int wtg_bv_sync(wtg_bv* B) {
  if (!B) return fail(WTG_ERR_INVALID, "null bitvector");
  return sync_and_check(B->stream, B->err.as<uint32_t>());
}

int wtg_bv_free(wtg_bv* B) {
  if (!B) return WTG_OK;
  cudaStream_t s = B->stream;
  bv_release(B->bv, s);
  B->words.release(s);
  B->err.release(s);
  B->qbuf.release(s);
  cudaStreamSynchronize(s);
  if (B->own_stream) cudaStreamDestroy(s);
  delete B;
  return WTG_OK;
}

int wtg_bv_rank_words(wtg_bv* B, uint64_t* nwords) {
  if (!B || !nwords) return fail(WTG_ERR_INVALID, "null argument");
  *nwords = rank_words_of(B->bv.size);
  return WTG_OK;
}

int wtg_bv_get_rank(wtg_bv* B, uint64_t* dst, uint64_t nwords) {
  if (!B || !dst) return fail(WTG_ERR_INVALID, "null argument");
  if (!(B->bv.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "rank support not built");
  if (nwords != rank_words_of(B->bv.size)) return fail(WTG_ERR_INVALID, "nwords mismatch");
  WTG_CK(cudaMemcpyAsync(dst, B->bv.rank.p, nwords * 8, cudaMemcpyDeviceToHost, B->stream));
  return sync_and_check(B->stream, B->err.as<uint32_t>());
}

int wtg_bv_select_info(wtg_bv* B, int t_b, uint64_t info[8]) {
  if (!B || !info || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  if (!(B->bv.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select support not built");
  fill_select_info(B->bv, t_b, info);
  return WTG_OK;
}

int wtg_bv_get_select(wtg_bv* B, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  if (!B || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  int rc = copy_select(B->bv, t_b, sb_words, desc, pool, B->stream);
  if (rc) return rc;
  return sync_and_check(B->stream, B->err.as<uint32_t>());
}

int wtg_bv_rank(wtg_bv* B, const uint64_t* idx, uint64_t nq, uint64_t* out) {
  if (!B || (nq && (!idx || !out))) return fail(WTG_ERR_INVALID, "null argument");
  const uint64_t* ins[1] = {idx};
  uint64_t* outs[1] = {out};
  return host_query(B->qbuf, B->stream, ins, 1, nq, outs, 1, B->err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_bv_rank(B->bv, din[0], nq, dout[0], B->stream);
                    });
}

int wtg_bv_select(wtg_bv* B, int t_b, const uint64_t* i, uint64_t nq, uint64_t* out) {
  if (!B || (t_b != 0 && t_b != 1) || (nq && (!i || !out))) return fail(WTG_ERR_INVALID, "bad argument");
  const uint64_t* ins[1] = {i};
  uint64_t* outs[1] = {out};
  return host_query(B->qbuf, B->stream, ins, 1, nq, outs, 1, B->err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_bv_select(B->bv, t_b, din[0], nq, dout[0], B->stream);
                    });
}

int wtg_bv_select_device(wtg_bv* B, int t_b, const uint64_t* d_i, uint64_t nq, uint64_t* d_out, void* stream) {
  if (!B || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  return launch_bv_select(B->bv, t_b, d_i, nq, d_out, (cudaStream_t)stream);
}

// ------------------------------------------------- suffix array and BWT

int wtg_suffix_array_device(const uint8_t* d_text, uint64_t n, int32_t* d_sa, uint8_t* d_bwt, void* stream,
                            int* rounds) {
  int rc;
  if (n && !d_text) return fail(WTG_ERR_INVALID, "null text");
  if ((rc = check_device())) return rc;
  return suffix_array_device(d_text, n, (uint32_t*)d_sa, d_bwt, rounds, (cudaStream_t)stream);
}

int wtg_bwt(const uint8_t* text, uint64_t n, uint8_t* bwt_out, int32_t* sa_out) {
  int rc;
  if (n && (!text || (!bwt_out && !sa_out))) return fail(WTG_ERR_INVALID, "null argument");
  if (n >= (1ull << 31)) return fail(WTG_ERR_INVALID, "suffix array: n must be below 2^31 (32-bit entries)");
  if (n == 0) return WTG_OK;
  if ((rc = check_device())) return rc;
  cudaStream_t s = nullptr;
  WTG_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf buf;
  const uint64_t text_bytes = (n + 15) / 16 * 16;
  rc = buf.ensure(text_bytes + 5 * n, s);  // text (padded), SA, BWT
  if (rc == WTG_OK) {
    uint8_t* d_text = buf.as<uint8_t>();
    uint32_t* d_sa = (uint32_t*)(d_text + text_bytes);
    uint8_t* d_bwt = (uint8_t*)(d_sa + n);
    cudaError_t e = cudaMemcpyAsync(d_text, text, n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "copy text");
    if (rc == WTG_OK) rc = suffix_array_device(d_text, n, d_sa, bwt_out ? d_bwt : nullptr, nullptr, s);
    if (rc == WTG_OK && sa_out) {
      e = cudaMemcpyAsync(sa_out, d_sa, n * 4, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) rc = cuda_fail(e, "copy SA");
    }
    if (rc == WTG_OK && bwt_out) {
      e = cudaMemcpyAsync(bwt_out, d_bwt, n, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) rc = cuda_fail(e, "copy BWT");
    }
    if (rc == WTG_OK) {
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_fail(e, "suffix array");
    }
  }
  buf.release(s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return rc;
}

int wtg_suffix_array(const uint8_t* text, uint64_t n, int32_t* sa_out) {
  if (n && !sa_out) return fail(WTG_ERR_INVALID, "null argument");
  return wtg_bwt(text, n, nullptr, sa_out);
}

// ------------------------------------------------------------ FM-index count

int wtg_fm_count(wtg_tree* T, const uint64_t* C, uint64_t sigma, const uint8_t* pat, const uint64_t* off,
                 uint64_t npat, uint64_t* out) {
  int rc;
  if (!T || !C || (npat && (!off || !out))) return fail(WTG_ERR_INVALID, "null argument");
  if (npat == 0) return WTG_OK;
  const uint64_t total = off[npat];
  if (total && !pat) return fail(WTG_ERR_INVALID, "null patterns");
  for (uint64_t p = 0; p < npat; ++p)
    if (off[p] > off[p + 1]) return fail(WTG_ERR_INVALID, "pattern offsets must not decrease");
  if (sigma == 0 || sigma > 256) return fail(WTG_ERR_INVALID, "sigma must be 1..256");
  TreeImpl& t = T->t;
  cudaStream_t s = t.stream;
  const uint64_t words = sigma + (npat + 1) + npat + (total + 7) / 8;
  if ((rc = t.qbuf.ensure(words * sizeof(uint64_t), s))) return rc;
  uint64_t* d = t.qbuf.as<uint64_t>();
  uint64_t* dC = d;
  uint64_t* dOff = dC + sigma;
  uint64_t* dOut = dOff + npat + 1;
  uint8_t* dPat = (uint8_t*)(dOut + npat);
  WTG_CK(cudaMemcpyAsync(dC, C, sigma * 8, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(dOff, off, (npat + 1) * 8, cudaMemcpyHostToDevice, s));
  if (total) WTG_CK(cudaMemcpyAsync(dPat, pat, total, cudaMemcpyHostToDevice, s));
  if ((rc = launch_fm_count(t, dC, sigma, dPat, dOff, npat, dOut, s))) return rc;
  WTG_CK(cudaMemcpyAsync(out, dOut, npat * 8, cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, t.err.as<uint32_t>());
}

int wtg_fm_count_device(wtg_tree* T, const uint64_t* d_C, uint64_t sigma, const uint8_t* d_pat,
                        const uint64_t* d_off, uint64_t npat, uint64_t* d_out, void* stream) {
  if (!T) return fail(WTG_ERR_INVALID, "null tree");
  return launch_fm_count(T->t, d_C, sigma, d_pat, d_off, npat, d_out, (cudaStream_t)stream);
}

// ------------------------------------------------ per-level and learned select

int wtg_tree_level_select(wtg_tree* T, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq,
                          uint64_t* out) {
  if (!T || (t_b != 0 && t_b != 1) || (nq && (!level || !k || !out))) return fail(WTG_ERR_INVALID, "bad argument");
  TreeImpl& t = T->t;
  const uint64_t* ins[2] = {level, k};
  uint64_t* outs[1] = {out};
  return host_query(t.qbuf, t.stream, ins, 2, nq, outs, 1, t.err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_level_select(t, t_b, din[0], din[1], nq, dout[0], t.stream);
                    });
}

int wtg_tree_level_select_device(wtg_tree* T, int t_b, const uint64_t* d_level, const uint64_t* d_k, uint64_t nq,
                                 uint64_t* d_out, void* stream) {
  if (!T || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  return launch_level_select(T->t, t_b, d_level, d_k, nq, d_out, (cudaStream_t)stream);
}

int wtg_lsel_build(wtg_tree* T, uint32_t segments, uint32_t samples, uint32_t max_window, wtg_lsel** out) {
  int rc;
  if (!T || !out) return fail(WTG_ERR_INVALID, "null argument");
  wtg_lsel* M = *out;
  bool fresh = false;
  if (!M) {
    M = new (std::nothrow) wtg_lsel();
    if (M) M->m = lsel_new();
    if (!M || !M->m) {
      delete M;
      return fail(WTG_ERR_OOM, "host allocation failed");
    }
    fresh = true;
  }
  rc = lsel_build(*M->m, T->t, segments, samples, max_window, T->t.stream);
  if (rc == WTG_OK) rc = sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
  if (rc != WTG_OK) {
    if (fresh) wtg_lsel_free(M);
    return rc;
  }
  *out = M;
  return WTG_OK;
}

int wtg_lsel_free(wtg_lsel* M) {
  if (!M) return WTG_OK;
  lsel_delete(M->m);  // waits for the device
  M->qbuf.release(nullptr);
  cudaDeviceSynchronize();
  delete M;
  return WTG_OK;
}

int wtg_lsel_info(wtg_lsel* M, uint64_t info[8]) {
  if (!M || !info) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl* t = lsel_tree(*M->m);
  return lsel_info(*M->m, info, t ? t->stream : nullptr);
}

int wtg_lsel_get_level(wtg_lsel* M, int t_b, int level, uint64_t lvl_info[4], uint32_t* rec, uint64_t nseg) {
  if (!M || !lvl_info) return fail(WTG_ERR_INVALID, "null argument");
  TreeImpl* t = lsel_tree(*M->m);
  return lsel_get_level(*M->m, t_b, level, lvl_info, rec, nseg, t ? t->stream : nullptr);
}

int wtg_lsel_query(wtg_lsel* M, int t_b, const uint64_t* level, const uint64_t* k, uint64_t nq, uint64_t* out) {
  if (!M || (t_b != 0 && t_b != 1) || (nq && (!level || !k || !out))) return fail(WTG_ERR_INVALID, "bad argument");
  TreeImpl* t = lsel_tree(*M->m);
  if (!t) return fail(WTG_ERR_INVALID, "the index's tree was freed");
  const uint64_t* ins[2] = {level, k};
  uint64_t* outs[1] = {out};
  return host_query(M->qbuf, t->stream, ins, 2, nq, outs, 1, t->err.as<uint32_t>(),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_lsel_query(*M->m, t_b, din[0], din[1], nq, dout[0], t->stream);
                    });
}

int wtg_lsel_query_device(wtg_lsel* M, int t_b, const uint64_t* d_level, const uint64_t* d_k, uint64_t nq,
                          uint64_t* d_out, void* stream) {
  if (!M || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  return launch_lsel_query(*M->m, t_b, d_level, d_k, nq, d_out, (cudaStream_t)stream);
}

// ------------------------------------------------------------ batched builds

int wtg_batch_plan(const uint64_t* lengths, uint64_t ntexts, int levels, uint32_t flags, void* stream,
                   wtg_batch** out) {
  int rc;
  if (!out || (ntexts && !lengths)) return fail(WTG_ERR_INVALID, "null argument");
  if ((rc = check_device())) return rc;
  wtg_batch* B = new (std::nothrow) wtg_batch();
  if (B) B->b = batch_new();
  if (!B || !B->b) {
    delete B;
    return fail(WTG_ERR_OOM, "host allocation failed");
  }
  cudaStream_t s = (cudaStream_t)stream;
  bool own = false;
  if (!s) {
    cudaError_t ce = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
      batch_delete(B->b);
      delete B;
      return cuda_fail(ce, "stream create");
    }
    own = true;
  }
  rc = batch_plan(*B->b, lengths, ntexts, levels, flags, s, own);
  if (rc != WTG_OK) {
    batch_delete(B->b);
    delete B;
    return rc;
  }
  *out = B;
  return WTG_OK;
}

int wtg_batch_input(wtg_batch* B, void** d_input, uint64_t* nbytes) {
  if (!B || !d_input || !nbytes) return fail(WTG_ERR_INVALID, "null argument");
  *d_input = batch_input(*B->b);
  *nbytes = batch_total_symbols(*B->b);
  return WTG_OK;
}

int wtg_batch_load(wtg_batch* B, const void* texts) {
  if (!B) return fail(WTG_ERR_INVALID, "null batch");
  const uint64_t nb = batch_total_symbols(*B->b);
  if (nb && !texts) return fail(WTG_ERR_INVALID, "null texts");
  if (nb) WTG_CK(cudaMemcpyAsync(batch_input(*B->b), texts, nb, cudaMemcpyHostToDevice, batch_stream(*B->b)));
  return WTG_OK;
}

int wtg_batch_set_shape(wtg_batch* B, int tile, int64_t whole_max, int symbols_per_thread) {
  if (!B) return fail(WTG_ERR_INVALID, "null batch");
  return batch_set_shape(*B->b, tile, whole_max, symbols_per_thread);
}

int wtg_batch_run(wtg_batch* B) {
  if (!B) return fail(WTG_ERR_INVALID, "null batch");
  return batch_run(*B->b);
}

int wtg_batch_sync(wtg_batch* B) {
  int rc;
  if (!B) return fail(WTG_ERR_INVALID, "null batch");
  uint32_t e = 0;
  if ((rc = batch_sync(*B->b, &e))) return rc;
  if (e == DERR_SELECT_OVERFLOW) return fail(WTG_ERR_CUDA, "a select pool exceeded its bound (inconsistent tables)");
  if (e) return fail(WTG_ERR_CUDA, "device reported error code " + std::to_string(e));
  return WTG_OK;
}

int wtg_batch_free(wtg_batch* B) {
  if (!B) return WTG_OK;
  batch_delete(B->b);
  delete B;
  return WTG_OK;
}

int wtg_batch_text_info(wtg_batch* B, uint64_t t, uint64_t info[8]) {
  if (!B || !info) return fail(WTG_ERR_INVALID, "null argument");
  return batch_text_info(*B->b, t, info);
}

int wtg_batch_select_info(wtg_batch* B, uint64_t t, int t_b, uint64_t info[8]) {
  if (!B || !info || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  return batch_select_info(*B->b, t, t_b, info);
}

int wtg_batch_get_bits(wtg_batch* B, uint64_t t, uint64_t* dst, uint64_t nwords) {
  if (!B || (nwords && !dst)) return fail(WTG_ERR_INVALID, "null argument");
  return batch_get(*B->b, t, 0, 0, dst, nwords);
}

int wtg_batch_get_rank(wtg_batch* B, uint64_t t, uint64_t* dst, uint64_t nwords) {
  if (!B || (nwords && !dst)) return fail(WTG_ERR_INVALID, "null argument");
  return batch_get(*B->b, t, 1, 0, dst, nwords);
}

int wtg_batch_get_select(wtg_batch* B, uint64_t t, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  int rc;
  if (!B || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  uint64_t si[8];
  if ((rc = batch_select_info(*B->b, t, t_b, si))) return rc;
  if ((si[6] && !sb_words) || (si[4] && !desc) || (si[7] && !pool)) return fail(WTG_ERR_INVALID, "null argument");
  if ((rc = batch_get(*B->b, t, 2, t_b, sb_words, si[6]))) return rc;
  if ((rc = batch_get(*B->b, t, 3, t_b, desc, si[4]))) return rc;
  return batch_get(*B->b, t, 4, t_b, pool, si[7]);
}

int wtg_batch_shape(wtg_batch* B, int* tile, int64_t* whole_max, int* symbols_per_thread, uint64_t* whole_texts,
                    float ms[8]) {
  if (!B || !tile || !whole_max || !symbols_per_thread || !whole_texts || !ms)
    return fail(WTG_ERR_INVALID, "null argument");
  return batch_shape(*B->b, tile, whole_max, symbols_per_thread, whole_texts, ms, 8);
}

// ------------------------------------------------ Huffman-shaped trees

static int huff_common(wtg_huff* H, const uint8_t* d_text, uint64_t n, uint32_t flags) {
  int rc = huff_build(*H->h, d_text, n, flags);
  if (rc) return rc;
  return sync_and_check(huff_stream(*H->h), huff_err(*H->h));
}

int wtg_huff_build(const uint8_t* text, uint64_t n, uint32_t flags, wtg_huff** out) {
  int rc;
  if (!out || (!text && n)) return fail(WTG_ERR_INVALID, "null argument");
  *out = nullptr;
  if ((rc = check_device())) return rc;
  wtg_huff* H = new (std::nothrow) wtg_huff();
  if (!H || !(H->h = huff_new())) {
    delete H;
    return fail(WTG_ERR_OOM, "host allocation failed");
  }
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    huff_delete(H->h);
    delete H;
    return cuda_fail(e, "cudaStreamCreate");
  }
  huff_set_stream(*H->h, s, true);
  DevBuf& t = huff_text(*H->h);
  rc = t.ensure(n + 16, s);
  if (rc == WTG_OK && n) {
    const cudaError_t ce = cudaMemcpyAsync(t.p, text, n, cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaMemcpyAsync(text)");
  }
  if (rc == WTG_OK) rc = huff_common(H, t.as<uint8_t>(), n, flags);
  if (rc != WTG_OK) {
    wtg_huff_free(H);
    return rc;
  }
  *out = H;
  return WTG_OK;
}

int wtg_huff_build_device(const uint8_t* d_text, uint64_t n, uint32_t flags, void* stream, wtg_huff** out) {
  int rc;
  if (!out || (!d_text && n)) return fail(WTG_ERR_INVALID, "null argument");
  *out = nullptr;
  if ((rc = check_device())) return rc;
  wtg_huff* H = new (std::nothrow) wtg_huff();
  if (!H || !(H->h = huff_new())) {
    delete H;
    return fail(WTG_ERR_OOM, "host allocation failed");
  }
  huff_set_stream(*H->h, (cudaStream_t)stream, false);
  if ((rc = huff_common(H, d_text, n, flags))) {
    wtg_huff_free(H);
    return rc;
  }
  *out = H;
  return WTG_OK;
}

int wtg_huff_free(wtg_huff* H) {
  if (!H) return WTG_OK;
  huff_delete(H->h);
  delete H;
  return WTG_OK;
}

int wtg_huff_info(wtg_huff* H, uint64_t info[5]) {
  if (!H || !info) return fail(WTG_ERR_INVALID, "null argument");
  return huff_info(*H->h, info);
}

int wtg_huff_get_bits(wtg_huff* H, uint64_t* dst, uint64_t nwords) {
  if (!H || (!dst && nwords)) return fail(WTG_ERR_INVALID, "null argument");
  uint64_t info[5];
  huff_info(*H->h, info);
  if (nwords != (info[2] + 63) / 64) return fail(WTG_ERR_INVALID, "nwords does not match the tree");
  cudaStream_t s = huff_stream(*H->h);
  if (nwords) WTG_CK(cudaMemcpyAsync(dst, huff_bits(*H->h), nwords * 8, cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, huff_err(*H->h));
}

int wtg_huff_get_tree(wtg_huff* H, uint64_t* nodes, uint64_t* leaves, uint64_t* paths) {
  if (!H || !nodes || !leaves || !paths) return fail(WTG_ERR_INVALID, "null argument");
  return huff_tree(*H->h, nodes, leaves, paths);
}

int wtg_huff_get_rank(wtg_huff* H, uint64_t* dst, uint64_t nwords) {
  if (!H || !dst) return fail(WTG_ERR_INVALID, "null argument");
  uint64_t info[5];
  huff_info(*H->h, info);
  if (!info[4]) return fail(WTG_ERR_INVALID, "rank support not built");
  if (nwords != info[4]) return fail(WTG_ERR_INVALID, "nwords mismatch");
  cudaStream_t s = huff_stream(*H->h);
  WTG_CK(cudaMemcpyAsync(dst, huff_bv(*H->h).rank.p, nwords * 8, cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, huff_err(*H->h));
}

int wtg_huff_select_info(wtg_huff* H, int t_b, uint64_t info[8]) {
  if (!H || !info || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  BvSupport& bv = huff_bv(*H->h);
  if (!(bv.flags & (t_b ? WTG_SELECT1 : WTG_SELECT0))) return fail(WTG_ERR_INVALID, "select support not built");
  fill_select_info(bv, t_b, info);
  return WTG_OK;
}

int wtg_huff_get_select(wtg_huff* H, int t_b, uint64_t* sb_words, uint64_t* desc, uint64_t* pool) {
  if (!H || (t_b != 0 && t_b != 1)) return fail(WTG_ERR_INVALID, "bad argument");
  int rc = copy_select(huff_bv(*H->h), t_b, sb_words, desc, pool, huff_stream(*H->h));
  if (rc) return rc;
  return sync_and_check(huff_stream(*H->h), huff_err(*H->h));
}

static int huff_host_query(wtg_huff* H, int what, const uint64_t* a, const uint64_t* b, uint64_t nq, uint64_t* out,
                           uint64_t* out2) {
  HuffImpl& h = *H->h;
  const uint64_t* ins[2] = {a, b};
  uint64_t* outs[2] = {out, out2};
  const int nin = (what == 1 || what == 2) ? 2 : 1, nout = what == 3 ? 2 : 1;
  cudaStream_t s = huff_stream(h);
  return host_query(huff_qbuf(h), s, ins, nin, nq, outs, nout, huff_err(h),
                    [&](const uint64_t** din, uint64_t** dout) {
                      return launch_huff_query(h, what, din[0], nin > 1 ? din[1] : nullptr, nq, dout[0],
                                               nout > 1 ? dout[1] : nullptr, s);
                    });
}

int wtg_huff_access(wtg_huff* H, const uint64_t* idx, uint64_t nq, uint64_t* out) {
  if (!H || (nq && (!idx || !out))) return fail(WTG_ERR_INVALID, "null argument");
  return huff_host_query(H, 0, idx, nullptr, nq, out, nullptr);
}

int wtg_huff_rank(wtg_huff* H, const uint64_t* idx, const uint64_t* sym, uint64_t nq, uint64_t* out) {
  if (!H || (nq && (!idx || !sym || !out))) return fail(WTG_ERR_INVALID, "null argument");
  return huff_host_query(H, 1, idx, sym, nq, out, nullptr);
}

int wtg_huff_select(wtg_huff* H, const uint64_t* i, const uint64_t* sym, uint64_t nq, uint64_t* out) {
  if (!H || (nq && (!i || !sym || !out))) return fail(WTG_ERR_INVALID, "null argument");
  return huff_host_query(H, 2, i, sym, nq, out, nullptr);
}

int wtg_huff_inverse_select(wtg_huff* H, const uint64_t* idx, uint64_t nq, uint64_t* rank_out, uint64_t* sym_out) {
  if (!H || (nq && (!idx || !rank_out || !sym_out))) return fail(WTG_ERR_INVALID, "null argument");
  return huff_host_query(H, 3, idx, nullptr, nq, rank_out, sym_out);
}

int wtg_huff_fm_count(wtg_huff* H, const uint64_t* C, const uint8_t* pat, const uint64_t* off, uint64_t npat,
                      uint64_t* out) {
  int rc;
  if (!H || !C || (npat && (!off || !out))) return fail(WTG_ERR_INVALID, "null argument");
  if (npat == 0) return WTG_OK;
  const uint64_t total = off[npat];
  if (total && !pat) return fail(WTG_ERR_INVALID, "null patterns");
  for (uint64_t p = 0; p < npat; ++p)
    if (off[p] > off[p + 1]) return fail(WTG_ERR_INVALID, "pattern offsets must not decrease");
  HuffImpl& h = *H->h;
  cudaStream_t s = huff_stream(h);
  DevBuf& q = huff_qbuf(h);
  const uint64_t words = 256 + (npat + 1) + npat + (total + 7) / 8;
  if ((rc = q.ensure(words * sizeof(uint64_t), s))) return rc;
  uint64_t* dC = q.as<uint64_t>();
  uint64_t* dOff = dC + 256;
  uint64_t* dOut = dOff + npat + 1;
  uint8_t* dPat = (uint8_t*)(dOut + npat);
  WTG_CK(cudaMemcpyAsync(dC, C, 256 * 8, cudaMemcpyHostToDevice, s));
  WTG_CK(cudaMemcpyAsync(dOff, off, (npat + 1) * 8, cudaMemcpyHostToDevice, s));
  if (total) WTG_CK(cudaMemcpyAsync(dPat, pat, total, cudaMemcpyHostToDevice, s));
  if ((rc = launch_huff_fm_count(h, dC, dPat, dOff, npat, dOut, s))) return rc;
  WTG_CK(cudaMemcpyAsync(out, dOut, npat * 8, cudaMemcpyDeviceToHost, s));
  return sync_and_check(s, huff_err(h));
}

int wtg_huff_fm_count_device(wtg_huff* H, const uint64_t* d_C, const uint8_t* d_pat, const uint64_t* d_off,
                             uint64_t npat, uint64_t* d_out, void* stream) {
  if (!H || !d_C || (npat && (!d_off || !d_out))) return fail(WTG_ERR_INVALID, "null argument");
  if (npat == 0) return WTG_OK;
  return launch_huff_fm_count(*H->h, d_C, d_pat, d_off, npat, d_out, (cudaStream_t)stream);
}

// ------------------------------------------------ sdsl serialize() streams

int wtg_tree_serialize(wtg_tree* T, void* dst, uint64_t cap, uint64_t* len) {
  if (!T || !len) return fail(WTG_ERR_INVALID, "null argument");
  int rc = tree_serialize(T->t, (uint8_t*)dst, cap, len);
  if (rc) return rc;
  return dst ? sync_and_check(T->t.stream, T->t.err.as<uint32_t>()) : WTG_OK;
}

int wtg_tree_sigma(wtg_tree* T, uint64_t* sigma) {
  if (!T || !sigma) return fail(WTG_ERR_INVALID, "null argument");
  int rc = tree_leaf_count(T->t, sigma, T->t.stream);
  if (rc) return rc;
  return sync_and_check(T->t.stream, T->t.err.as<uint32_t>());
}

int wtg_bv_serialize(wtg_bv* B, uint32_t part, void* dst, uint64_t cap, uint64_t* len) {
  if (!B || !len) return fail(WTG_ERR_INVALID, "null argument");
  int rc = bv_serialize(B->bv, part, (uint8_t*)dst, cap, len, B->stream);
  if (rc) return rc;
  return dst ? sync_and_check(B->stream, B->err.as<uint32_t>()) : WTG_OK;
}

// ------------------------------------------------ failure handling knobs

int wtg_set_wait_limits(uint32_t lookback_spins, uint32_t mbarrier_tries) {
  int rc;
  if ((rc = check_device())) return rc;
  const uint32_t lim[2] = {lookback_spins ? lookback_spins : LB_SPIN_LIMIT,
                           mbarrier_tries ? mbarrier_tries : MBAR_SPIN_LIMIT};
  if ((rc = set_wait_limits_build(lim))) return rc;
  if ((rc = set_wait_limits_batch(lim))) return rc;
  if ((rc = set_wait_limits_bitvec(lim))) return rc;
  return set_wait_limits_core(lim);
}

int wtg_test_fail_alloc(int64_t nth) {
  if (nth < 0) return fail(WTG_ERR_INVALID, "nth must be >= 0");
  test_arm_alloc_failure(nth);
  return WTG_OK;
}

int wtg_test_stall_lookback(int on) {
  test_arm_lookback_stall(on);
  return WTG_OK;
}

// ------------------------------------------------------------------ helpers

int wtg_remap_alphabet(void* seq, uint64_t n, int elem_bytes, uint64_t* sigma_out) {
  int rc;
  if (!sigma_out || (!seq && n)) return fail(WTG_ERR_INVALID, "null argument");
  if (elem_bytes != 1 && elem_bytes != 2 && elem_bytes != 4 && elem_bytes != 8)
    return fail(WTG_ERR_INVALID, "elem_bytes must be 1, 2, 4 or 8");
  if ((rc = check_device())) return rc;
  cudaStream_t s;
  WTG_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf d, tmp, scan_tmp, err;
  rc = d.ensure(n * elem_bytes, s);
  if (!rc) rc = err.ensure(sizeof(uint32_t), s);
  if (!rc) {
    cudaError_t ce = cudaMemsetAsync(err.p, 0, sizeof(uint32_t), s);
    if (ce == cudaSuccess && n) ce = cudaMemcpyAsync(d.p, seq, n * elem_bytes, cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "copy sequence");
  }
  if (!rc) rc = remap_alphabet_device(d.p, n, elem_bytes, sigma_out, tmp, scan_tmp, err.as<uint32_t>(), s);
  if (!rc && n) {
    cudaError_t ce = cudaMemcpyAsync(seq, d.p, n * elem_bytes, cudaMemcpyDeviceToHost, s);
    if (ce != cudaSuccess) rc = cuda_fail(ce, "copy sequence back");
  }
  if (!rc) rc = sync_and_check(s, err.as<uint32_t>());
  d.release(s);
  tmp.release(s);
  scan_tmp.release(s);
  err.release(s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return rc;
}

}  // extern "C"
