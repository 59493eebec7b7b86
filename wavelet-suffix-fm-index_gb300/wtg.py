"""Python binding of libwtg (include/wtg.h): GPU wavelet-tree construction,
rank_support_v / select_support_mcl supports and wt_int queries.

Mirrors the reference's interface for this path:
  * WT(s, sigma)                -> (nodes, bits) like WT(symbol*, n, sigma)
                                   (wavelet/levelWT/WT.h:43)
  * WaveletTree(seq, max_level) -> sdsl::wt_int<> (wt_int/wt_int_par.hpp:368),
                                   with access ([]), rank, select,
                                   inverse_select
  * BitVectorSupport(words, n)  -> rank_support_v<1> + select_support_mcl<1>/<0>
                                   over a bit_vector
Every call runs CUDA kernels through the C ABI; there is no CPU path.  If the
library cannot be loaded, or no GPU is usable, calls raise WtgError.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwtg.so")

OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_RANGE = 0, 1, 2, 3, 4, 5
RANK, SELECT1, SELECT0, ALL = 1, 2, 4, 7
NONE = np.uint64(0xFFFFFFFFFFFFFFFF)

u64 = ctypes.c_uint64
vp = ctypes.c_void_p
i32 = ctypes.c_int


class WtgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"wtg error {code}: {msg}")
        self.code = code


_lib = None


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("wtg_build_lib", os.path.join(HERE, "build_lib.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build()


_SIGS = {
    "wtg_last_error": ([], ctypes.c_char_p),
    "wtg_version": ([], i32),
    "wtg_launch_count": ([], u64),
    "wtg_tree_build": ([vp, u64, i32, i32, ctypes.c_uint32, vp], i32),
    "wtg_tree_build_device": ([vp, u64, i32, i32, ctypes.c_uint32, vp, vp], i32),
    "wtg_tree_build_out": ([vp, u64, i32, i32, ctypes.c_uint32, vp, vp, vp], i32),
    "wtg_tree_sync": ([vp], i32),
    "wtg_tree_free": ([vp], i32),
    "wtg_tree_info": ([vp, vp], i32),
    "wtg_tree_select_info": ([vp, i32, vp], i32),
    "wtg_tree_get_bits": ([vp, vp, u64], i32),
    "wtg_tree_get_nodes": ([vp, i32, u64, vp], i32),
    "wtg_tree_get_rank": ([vp, vp, u64], i32),
    "wtg_tree_get_select": ([vp, i32, vp, vp, vp], i32),
    "wtg_tree_device_ptrs": ([vp, vp], i32),
    "wtg_query_access": ([vp, vp, u64, vp], i32),
    "wtg_query_rank": ([vp, vp, vp, u64, vp], i32),
    "wtg_query_inverse_select": ([vp, vp, u64, vp, vp], i32),
    "wtg_query_select": ([vp, vp, vp, u64, vp], i32),
    "wtg_query_access_device": ([vp, vp, u64, vp, vp], i32),
    "wtg_query_rank_device": ([vp, vp, vp, u64, vp, vp], i32),
    "wtg_suffix_array": ([vp, u64, vp], i32),
    "wtg_bwt": ([vp, u64, vp, vp], i32),
    "wtg_suffix_array_device": ([vp, u64, vp, vp, vp, vp], i32),
    "wtg_query_lex_count": ([vp, vp, vp, vp, u64, vp, vp, vp], i32),
    "wtg_query_lex_smaller_count": ([vp, vp, vp, u64, vp, vp], i32),
    "wtg_query_range_search_2d": ([vp, vp, vp, vp, vp, u64, vp, u64, vp, vp], i32),
    "wtg_query_interval_symbols": ([vp, vp, vp, u64, vp, u64, vp, vp, vp], i32),
    "wtg_query_expand": ([vp, vp, u64, vp, vp], i32),
    "wtg_query_expand_ranges": ([vp, vp, vp, u64, vp, vp], i32),
    "wtg_query_lex_count_device": ([vp, vp, vp, vp, u64, vp, vp, vp, vp], i32),
    "wtg_query_range_count_device": ([vp, vp, vp, vp, vp, u64, vp, vp], i32),
    "wtg_bv_build": ([vp, u64, ctypes.c_uint32, vp], i32),
    "wtg_bv_build_device": ([vp, u64, ctypes.c_uint32, vp, vp], i32),
    "wtg_bv_sync": ([vp], i32),
    "wtg_bv_free": ([vp], i32),
    "wtg_bv_rank_words": ([vp, vp], i32),
    "wtg_bv_get_rank": ([vp, vp, u64], i32),
    "wtg_bv_select_info": ([vp, i32, vp], i32),
    "wtg_bv_get_select": ([vp, i32, vp, vp, vp], i32),
    "wtg_bv_rank": ([vp, vp, u64, vp], i32),
    "wtg_bv_select": ([vp, i32, vp, u64, vp], i32),
    "wtg_bv_select_device": ([vp, i32, vp, u64, vp, vp], i32),
    "wtg_tree_level_select": ([vp, i32, vp, vp, u64, vp], i32),
    "wtg_tree_level_select_device": ([vp, i32, vp, vp, u64, vp, vp], i32),
    "wtg_lsel_build": ([vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp], i32),
    "wtg_lsel_free": ([vp], i32),
    "wtg_lsel_info": ([vp, vp], i32),
    "wtg_lsel_get_level": ([vp, i32, i32, vp, vp, u64], i32),
    "wtg_lsel_query": ([vp, i32, vp, vp, u64, vp], i32),
    "wtg_lsel_query_device": ([vp, i32, vp, vp, u64, vp, vp], i32),
    "wtg_fm_count": ([vp, vp, u64, vp, vp, u64, vp], i32),
    "wtg_fm_count_device": ([vp, vp, u64, vp, vp, u64, vp, vp], i32),
    "wtg_batch_plan": ([vp, u64, i32, ctypes.c_uint32, vp, vp], i32),
    "wtg_batch_input": ([vp, vp, vp], i32),
    "wtg_batch_load": ([vp, vp], i32),
    "wtg_batch_run": ([vp], i32),
    "wtg_batch_set_shape": ([vp, i32, ctypes.c_int64, i32], i32),
    "wtg_batch_sync": ([vp], i32),
    "wtg_batch_free": ([vp], i32),
    "wtg_batch_text_info": ([vp, u64, vp], i32),
    "wtg_batch_select_info": ([vp, u64, i32, vp], i32),
    "wtg_batch_get_bits": ([vp, u64, vp, u64], i32),
    "wtg_batch_get_rank": ([vp, u64, vp, u64], i32),
    "wtg_batch_get_select": ([vp, u64, i32, vp, vp, vp], i32),
    "wtg_batch_shape": ([vp, vp, vp, vp, vp, vp], i32),
    "wtg_remap_alphabet": ([vp, u64, i32, vp], i32),
    "wtg_rank_build_noalloc": ([vp, u64, vp, vp], i32),
    "wtg_profile_enable": ([i32], i32),
    "wtg_profile_read": ([vp, vp], i32),
    "wtg_huff_build": ([vp, u64, ctypes.c_uint32, vp], i32),
    "wtg_huff_build_device": ([vp, u64, ctypes.c_uint32, vp, vp], i32),
    "wtg_huff_free": ([vp], i32),
    "wtg_huff_info": ([vp, vp], i32),
    "wtg_huff_get_bits": ([vp, vp, u64], i32),
    "wtg_huff_get_tree": ([vp, vp, vp, vp], i32),
    "wtg_huff_get_rank": ([vp, vp, u64], i32),
    "wtg_huff_select_info": ([vp, i32, vp], i32),
    "wtg_huff_get_select": ([vp, i32, vp, vp, vp], i32),
    "wtg_huff_access": ([vp, vp, u64, vp], i32),
    "wtg_huff_rank": ([vp, vp, vp, u64, vp], i32),
    "wtg_huff_select": ([vp, vp, vp, u64, vp], i32),
    "wtg_huff_inverse_select": ([vp, vp, u64, vp, vp], i32),
    "wtg_huff_fm_count": ([vp, vp, vp, vp, u64, vp], i32),
    "wtg_huff_fm_count_device": ([vp, vp, vp, vp, u64, vp, vp], i32),
    "wtg_tree_serialize": ([vp, vp, u64, vp], i32),
    "wtg_tree_sigma": ([vp, vp], i32),
    "wtg_bv_serialize": ([vp, ctypes.c_uint32, vp, u64, vp], i32),
    "wtg_set_wait_limits": ([ctypes.c_uint32, ctypes.c_uint32], i32),
    "wtg_test_fail_alloc": ([ctypes.c_int64], i32),
    "wtg_test_stall_lookback": ([i32], i32),
}


def lib():
    """The loaded libwtg (built on first use when missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _ck(rc):
    if rc != OK:
        msg = lib().wtg_last_error()
        raise WtgError(rc, msg.decode() if msg else "")


def launch_count():
    return int(lib().wtg_launch_count())


def set_wait_limits(lookback_spins=0, mbarrier_tries=0):
    """Limits of the bounded device waits on the current device (0: default)."""
    _ck(lib().wtg_set_wait_limits(int(lookback_spins), int(mbarrier_tries)))


def inject_alloc_failure(nth):
    """Test hook: the nth next device allocation fails with ERR_OOM (0 disarms)."""
    _ck(lib().wtg_test_fail_alloc(int(nth)))


def inject_lookback_stall(on=True):
    """Test hook: the next rank/select pass over a caller bitvector never
    publishes its first tile, so its look-back waits run out (ERR_TIMEOUT)."""
    _ck(lib().wtg_test_stall_lookback(1 if on else 0))


PROF_CLASSES = ("level", "level_last", "hist", "tables", "bvpass", "select")


def profile_enable(on=True):
    _ck(lib().wtg_profile_enable(1 if on else 0))


def profile_read():
    """{class: (launches, total device ms)} recorded since the last read."""
    n = np.zeros(len(PROF_CLASSES), dtype=np.uint64)
    ms = np.zeros(len(PROF_CLASSES), dtype=np.float64)
    _ck(lib().wtg_profile_read(_p(n), _p(ms)))
    return {c: (int(n[i]), float(ms[i])) for i, c in enumerate(PROF_CLASSES)}


def levels_for_sigma(sigma):
    """max(1, log2Up(sigma)) (wavelet/levelWT/WT.C:53)."""
    a, b = 0, int(sigma) - 1
    while b > 0:
        b >>= 1
        a += 1
    return max(1, a)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


class _SelectTables:
    """select_support_mcl<t_b> in the flat packed layout (see include/wtg.h)."""

    def __init__(self, info, sb_words, desc, pool):
        (self.size, self.arg_cnt, self.logn, self.logn4, self.nsb, self.has_long,
         self.sb_nwords, self.pool_nwords) = [int(x) for x in info]
        self.sb_words, self.desc, self.pool = sb_words, desc, pool


class WaveletTree:
    """Wavelet tree over n symbols built on the GPU (sdsl::wt_int<> semantics
    with levels = max_level; the level bits equal levelWT's WT() for
    levels = max(1, log2Up(sigma)))."""

    def __init__(self, seq=None, levels=0, flags=ALL, _handle=None):
        self.h = vp()
        if _handle is not None:
            self.h = _handle
        else:
            seq = np.ascontiguousarray(seq)
            if seq.dtype.itemsize not in (1, 2, 4, 8) or seq.dtype.kind != "u":
                raise ValueError("sequence must be an unsigned integer array of 1, 2, 4 or 8 byte symbols")
            _ck(lib().wtg_tree_build(_p(seq), seq.size, seq.dtype.itemsize, int(levels), flags,
                                     ctypes.byref(self.h)))
        info = np.zeros(4, dtype=np.uint64)
        _ck(lib().wtg_tree_info(self.h, _p(info)))
        self.n, self.levels, self.bit_words, self.rank_words = [int(x) for x in info]
        self.flags = flags

    @classmethod
    def build_out(cls, seq, levels, flags, bits_ptr, rank_ptr, tree=None):
        """Build from host memory and copy the bits (and the rank table) to
        the host buffers at bits_ptr / rank_ptr while the build runs
        (wtg_tree_build_out); returns the tree for the remaining outputs."""
        seq = np.ascontiguousarray(seq)
        h = tree.h if tree is not None else vp()
        _ck(lib().wtg_tree_build_out(_p(seq), seq.size, seq.dtype.itemsize, int(levels), flags, vp(bits_ptr),
                                     vp(rank_ptr), ctypes.byref(h)))
        if tree is not None:
            tree.__init__(_handle=h, flags=flags)
            return tree
        return cls(_handle=h, flags=flags)

    @classmethod
    def from_device(cls, d_ptr, n, elem_bytes, levels, flags=ALL, stream=0, tree=None):
        """Build (or rebuild `tree`) from a device pointer on a CUDA stream."""
        h = tree.h if tree is not None else vp()
        _ck(lib().wtg_tree_build_device(vp(d_ptr), n, elem_bytes, levels, flags, vp(stream), ctypes.byref(h)))
        if tree is not None:
            tree.__init__(_handle=h, flags=flags)
            return tree
        return cls(_handle=h, flags=flags)

    def sync(self):
        _ck(lib().wtg_tree_sync(self.h))

    def free(self):
        if self.h:
            lib().wtg_tree_free(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # outputs in the reference layouts
    def bits(self):
        out = np.zeros(self.bit_words, dtype=np.uint64)
        _ck(lib().wtg_tree_get_bits(self.h, _p(out), out.size))
        return out

    def nodes(self, n_entries, index_bytes=8):
        out = np.zeros((n_entries, 5), dtype=np.uint32 if index_bytes == 4 else np.uint64)
        _ck(lib().wtg_tree_get_nodes(self.h, index_bytes, n_entries, _p(out)))
        return out

    def rank_table(self):
        out = np.zeros(self.rank_words, dtype=np.uint64)
        _ck(lib().wtg_tree_get_rank(self.h, _p(out), out.size))
        return out

    def select_tables(self, t_b):
        info = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_tree_select_info(self.h, t_b, _p(info)))
        sb = np.zeros(max(int(info[6]), 1), dtype=np.uint64)
        desc = np.zeros(max(int(info[4]), 1), dtype=np.uint64)
        pool = np.zeros(max(int(info[7]), 1), dtype=np.uint64)
        _ck(lib().wtg_tree_get_select(self.h, t_b, _p(sb), _p(desc), _p(pool)))
        return _SelectTables(info, sb[: int(info[6])], desc[: int(info[4])], pool[: int(info[7])])

    def device_ptrs(self):
        out = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_tree_device_ptrs(self.h, _p(out)))
        return [int(x) for x in out]

    # wt_int queries (batched)
    def access(self, idx):
        idx = _u64(idx)
        out = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_query_access(self.h, _p(idx), idx.size, _p(out)))
        return out

    def __getitem__(self, i):
        return int(self.access(np.array([i]))[0])

    def rank(self, idx, sym):
        idx, sym = _u64(idx), _u64(sym)
        out = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_query_rank(self.h, _p(idx), _p(sym), idx.size, _p(out)))
        return out

    def inverse_select(self, idx):
        idx = _u64(idx)
        r = np.zeros(idx.size, dtype=np.uint64)
        c = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_query_inverse_select(self.h, _p(idx), idx.size, _p(r), _p(c)))
        return r, c

    def select(self, i, sym):
        i, sym = _u64(i), _u64(sym)
        out = np.zeros(i.size, dtype=np.uint64)
        _ck(lib().wtg_query_select(self.h, _p(i), _p(sym), i.size, _p(out)))
        return out

    # wt_int range queries (batched; UINT64_MAX answers for invalid bounds)
    def lex_count(self, i, j, c):
        """Rows (rank(i, c), symbols < c in [i, j), symbols > c in [i, j))."""
        i, j, c = _u64(i), _u64(j), _u64(c)
        out = np.zeros((3, i.size), dtype=np.uint64)
        _ck(lib().wtg_query_lex_count(self.h, _p(i), _p(j), _p(c), i.size, _p(out[0]), _p(out[1]), _p(out[2])))
        return out.T.copy()

    def lex_smaller_count(self, i, c):
        """Rows (rank(i, c), symbols < c in [0, i))."""
        i, c = _u64(i), _u64(c)
        out = np.zeros((2, i.size), dtype=np.uint64)
        _ck(lib().wtg_query_lex_smaller_count(self.h, _p(i), _p(c), i.size, _p(out[0]), _p(out[1])))
        return out.T.copy()

    def range_count(self, lb, rb, vlb, vrb):
        """range_search_2d(lb, rb, vlb, vrb, report=false) counts."""
        lb, rb, vlb, vrb = _u64(lb), _u64(rb), _u64(vlb), _u64(vrb)
        cnt = np.zeros(lb.size, dtype=np.uint64)
        _ck(lib().wtg_query_range_search_2d(self.h, _p(lb), _p(rb), _p(vlb), _p(vrb), lb.size, _p(cnt), 0,
                                            None, None))
        return cnt

    def range_search_2d(self, lb, rb, vlb, vrb, cap=None):
        """range_search_2d with report: (counts, offsets, positions, values);
        query q's points are positions/values[offsets[q]:offsets[q+1]]."""
        cnt = self.range_count(lb, rb, vlb, vrb)
        lb, rb, vlb, vrb = _u64(lb), _u64(rb), _u64(vlb), _u64(vrb)
        valid = np.where(cnt == NONE, np.uint64(0), cnt)
        off = np.concatenate([[0], np.cumsum(valid.astype(np.int64))]).astype(np.int64)
        total = int(off[-1]) if cap is None else min(int(off[-1]), int(cap))
        pos = np.zeros(max(total, 1), dtype=np.uint64)
        val = np.zeros(max(total, 1), dtype=np.uint64)
        if total:
            _ck(lib().wtg_query_range_search_2d(self.h, _p(lb), _p(rb), _p(vlb), _p(vrb), lb.size, _p(cnt), total,
                                                _p(pos), _p(val)))
        return cnt, off, pos[:total], val[:total]

    def interval_symbols(self, i, j):
        """interval_symbols: (k, offsets, symbols, rank(i, c), rank(j, c));
        query q's symbols are [offsets[q]:offsets[q+1]]."""
        i, j = _u64(i), _u64(j)
        k = np.zeros(i.size, dtype=np.uint64)
        _ck(lib().wtg_query_interval_symbols(self.h, _p(i), _p(j), i.size, _p(k), 0, None, None, None))
        valid = np.where(k == NONE, np.uint64(0), k)
        off = np.concatenate([[0], np.cumsum(valid.astype(np.int64))]).astype(np.int64)
        total = int(off[-1])
        cs, ri, rj = (np.zeros(max(total, 1), dtype=np.uint64) for _ in range(3))
        if total:
            _ck(lib().wtg_query_interval_symbols(self.h, _p(i), _p(j), i.size, _p(k), total, _p(cs), _p(ri),
                                                 _p(rj)))
        return k, off, cs[:total], ri[:total], rj[:total]

    def expand(self, nodes):
        """Children of nodes (rows (offset, size, level, sym)): (left, right)."""
        v = _u64(nodes).reshape(-1, 4)
        left, right = np.zeros_like(v), np.zeros_like(v)
        _ck(lib().wtg_query_expand(self.h, _p(v), v.shape[0], _p(left), _p(right)))
        return left, right

    def expand_ranges(self, node, ranges):
        """Closed ranges [s, e] (rows) of node v mapped to its children."""
        v, r = _u64(node), _u64(ranges).reshape(-1, 2)
        left, right = np.zeros_like(r), np.zeros_like(r)
        _ck(lib().wtg_query_expand_ranges(self.h, _p(v), _p(r), r.shape[0], _p(left), _p(right)))
        return left, right

    def lex_count_device(self, d_i, d_j, d_c, nq, d_rank, d_smaller, d_greater, stream=0):
        _ck(lib().wtg_query_lex_count_device(self.h, vp(d_i), vp(d_j), vp(d_c), nq, vp(d_rank), vp(d_smaller),
                                             vp(d_greater), vp(stream)))

    def range_count_device(self, d_lb, d_rb, d_vlb, d_vrb, nq, d_count, stream=0):
        _ck(lib().wtg_query_range_count_device(self.h, vp(d_lb), vp(d_rb), vp(d_vlb), vp(d_vrb), nq, vp(d_count),
                                               vp(stream)))

    def access_device(self, d_idx, nq, d_out, stream=0):
        _ck(lib().wtg_query_access_device(self.h, vp(d_idx), nq, vp(d_out), vp(stream)))

    def rank_device(self, d_idx, d_sym, nq, d_out, stream=0):
        _ck(lib().wtg_query_rank_device(self.h, vp(d_idx), vp(d_sym), nq, vp(d_out), vp(stream)))

    def serialize(self):
        """sdsl wt_int<>::serialize stream of the tree (uint8 array)."""
        n = ctypes.c_uint64(0)
        _ck(lib().wtg_tree_serialize(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.uint8)
        _ck(lib().wtg_tree_serialize(self.h, _p(out), out.size, ctypes.byref(n)))
        return out

    def sigma(self):
        """wt_int's sigma: the number of non-empty leaves."""
        v = ctypes.c_uint64(0)
        _ck(lib().wtg_tree_sigma(self.h, ctypes.byref(v)))
        return int(v.value)

    def level_select(self, level, k, t_b=1):
        """Position inside level `level` of its k-th one (t_b=1) or zero
        (t_b=0) through select_support_mcl (wt_int_par.hpp:651-656)."""
        level, k = _u64(level), _u64(k)
        out = np.zeros(k.size, dtype=np.uint64)
        _ck(lib().wtg_tree_level_select(self.h, t_b, _p(level), _p(k), k.size, _p(out)))
        return out

    def level_select_device(self, t_b, d_level, d_k, nq, d_out, stream=0):
        _ck(lib().wtg_tree_level_select_device(self.h, t_b, vp(d_level), vp(d_k), nq, vp(d_out), vp(stream)))


def WT(s, sigma, index_bytes=4):
    """levelWT's WT(s, n, sigma): returns (nodes [2*sigma, 5], bits) with
    levels = max(1, log2Up(sigma)) (wavelet/levelWT/WT.C:43-227)."""
    t = WaveletTree(s, levels=levels_for_sigma(sigma), flags=0)
    try:
        return t.nodes(2 * int(sigma), index_bytes), t.bits()
    finally:
        t.free()


class BitVectorSupport:
    """rank_support_v<1> and select_support_mcl<1>/<0> over the first
    size_bits bits of a bit_vector given as uint64 words."""

    def __init__(self, words, size_bits, flags=ALL):
        self.h = vp()
        words = _u64(words)
        self.size = int(size_bits)
        self.flags = flags
        _ck(lib().wtg_bv_build(_p(words), self.size, flags, ctypes.byref(self.h)))

    def free(self):
        if self.h:
            lib().wtg_bv_free(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def rank_table(self):
        n = ctypes.c_uint64(0)
        _ck(lib().wtg_bv_rank_words(self.h, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.uint64)
        _ck(lib().wtg_bv_get_rank(self.h, _p(out), out.size))
        return out

    def select_tables(self, t_b):
        info = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_bv_select_info(self.h, t_b, _p(info)))
        sb = np.zeros(max(int(info[6]), 1), dtype=np.uint64)
        desc = np.zeros(max(int(info[4]), 1), dtype=np.uint64)
        pool = np.zeros(max(int(info[7]), 1), dtype=np.uint64)
        _ck(lib().wtg_bv_get_select(self.h, t_b, _p(sb), _p(desc), _p(pool)))
        return _SelectTables(info, sb[: int(info[6])], desc[: int(info[4])], pool[: int(info[7])])

    def rank(self, idx):
        idx = _u64(idx)
        out = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_bv_rank(self.h, _p(idx), idx.size, _p(out)))
        return out

    def serialize(self, part):
        """sdsl serialize() stream of one support: part RANK gives
        rank_support_v, SELECT1 / SELECT0 select_support_mcl<1> / <0>."""
        n = ctypes.c_uint64(0)
        _ck(lib().wtg_bv_serialize(self.h, part, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.uint8)
        _ck(lib().wtg_bv_serialize(self.h, part, _p(out), out.size, ctypes.byref(n)))
        return out

    def select(self, i, t_b=1):
        i = _u64(i)
        out = np.zeros(i.size, dtype=np.uint64)
        _ck(lib().wtg_bv_select(self.h, t_b, _p(i), i.size, _p(out)))
        return out


class LearnedSelect:
    """Learned select index over a tree's level bitvectors (include/wtg.h:
    wtg_lsel_build): per level and polarity, at most `segments` least-squares
    lines with exact error windows; answers equal WaveletTree.level_select."""

    def __init__(self, tree, segments=1024, samples=1024, max_window=1 << 16):
        self.h = vp()
        self.tree = tree  # the index reads the tree's device buffers
        _ck(lib().wtg_lsel_build(tree.h, segments, samples, max_window, ctypes.byref(self.h)))

    def free(self):
        if self.h:
            lib().wtg_lsel_free(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def info(self):
        a = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_lsel_info(self.h, _p(a)))
        keys = ("segments", "index_bytes", "fallback_segments", "max_window", "window_sum", "misses",
                "segments_param", "samples_param")
        return {k: int(v) for k, v in zip(keys, a)}

    def level_model(self, t_b, level):
        """({A, m, g, nseg}, records [nseg, 4] as (base, slope, dlo, dhi))."""
        li = np.zeros(4, dtype=np.uint64)
        _ck(lib().wtg_lsel_get_level(self.h, t_b, level, _p(li), None, 0))
        nseg = int(li[3])
        rec = np.zeros((max(nseg, 1), 4), dtype=np.uint32)
        _ck(lib().wtg_lsel_get_level(self.h, t_b, level, _p(li), _p(rec), nseg))
        meta = dict(zip(("A", "m", "g", "nseg"), (int(x) for x in li)))
        return meta, rec[:nseg]

    def select(self, level, k, t_b=1):
        level, k = _u64(level), _u64(k)
        out = np.zeros(k.size, dtype=np.uint64)
        _ck(lib().wtg_lsel_query(self.h, t_b, _p(level), _p(k), k.size, _p(out)))
        return out

    def select_device(self, t_b, d_level, d_k, nq, d_out, stream=0):
        _ck(lib().wtg_lsel_query_device(self.h, t_b, vp(d_level), vp(d_k), nq, vp(d_out), vp(stream)))


def suffix_array(text):
    """Suffix array of a byte text (int32, the order divsufsort gives)."""
    text = np.ascontiguousarray(text, dtype=np.uint8)
    sa = np.zeros(max(text.size, 1), dtype=np.int32)
    _ck(lib().wtg_suffix_array(_p(text), text.size, _p(sa)))
    return sa[: text.size]


def bwt(text, with_sa=False):
    """BWT of a byte text by fm-index/par/WT.C:38-41 (and its suffix array)."""
    text = np.ascontiguousarray(text, dtype=np.uint8)
    out = np.zeros(max(text.size, 1), dtype=np.uint8)
    sa = np.zeros(max(text.size, 1), dtype=np.int32) if with_sa else None
    _ck(lib().wtg_bwt(_p(text), text.size, _p(out), _p(sa) if with_sa else None))
    return (out[: text.size], sa[: text.size]) if with_sa else out[: text.size]


def suffix_array_device(d_text, n, d_sa=0, d_bwt=0, stream=0):
    """Device variant; returns the number of doubling rounds."""
    r = ctypes.c_int(0)
    _ck(lib().wtg_suffix_array_device(vp(d_text), n, vp(d_sa), vp(d_bwt), vp(stream), ctypes.byref(r)))
    return r.value


class FMIndex:
    """FM-index core over a BWT (fm-index/par/WT.C:33-45: the wavelet tree of
    s[SA[i]-1]): a GPU wavelet tree over the BWT's symbol codes
    (0..sigma-1), the C array, and backward-search counting on the GPU."""

    def __init__(self, bwt_codes, sigma):
        bwt_codes = np.ascontiguousarray(bwt_codes, dtype=np.uint8)
        self.n, self.sigma = bwt_codes.size, int(sigma)
        self.tree = WaveletTree(bwt_codes, levels=levels_for_sigma(self.sigma), flags=ALL)
        occ = self.tree.rank(np.full(self.sigma, self.n), np.arange(self.sigma))
        self.C = np.concatenate([[0], np.cumsum(occ)[:-1]]).astype(np.uint64)

    @classmethod
    def from_device(cls, d_codes, n, sigma, stream=0):
        """FM-index over a BWT already on the device (codes 0..sigma-1, u8)."""
        fm = cls.__new__(cls)
        fm.n, fm.sigma = int(n), int(sigma)
        fm.tree = WaveletTree.from_device(d_codes, n, 1, levels_for_sigma(fm.sigma), ALL, stream)
        fm.tree.sync()
        occ = fm.tree.rank(np.full(fm.sigma, fm.n), np.arange(fm.sigma))
        fm.C = np.concatenate([[0], np.cumsum(occ)[:-1]]).astype(np.uint64)
        return fm

    @classmethod
    def from_text(cls, text):
        """FM-index of a byte text, built as fm-index/par/WT.C:33-44 does:
        suffix array and BWT on the GPU, the BWT's bytes coded 0..sigma-1 in
        byte order, its wavelet tree.  Returns (index, byte -> code table)."""
        b = bwt(text)
        present = np.zeros(256, dtype=bool)
        present[np.unique(b)] = True
        code = np.cumsum(present).astype(np.int64) - 1
        fm = cls(code[b].astype(np.uint8), int(present.sum()))
        return fm, np.where(present, code, -1)

    @staticmethod
    def pack(patterns):
        """Concatenated codes and offsets of a list of code arrays."""
        off = np.zeros(len(patterns) + 1, dtype=np.uint64)
        off[1:] = np.cumsum([len(p) for p in patterns])
        pat = np.concatenate([np.asarray(p, dtype=np.uint8) for p in patterns]) if patterns else np.zeros(0, np.uint8)
        return pat, off

    def count(self, pat, off):
        pat = np.ascontiguousarray(pat, dtype=np.uint8)
        off = np.ascontiguousarray(off, dtype=np.uint64)
        out = np.zeros(off.size - 1, dtype=np.uint64)
        _ck(lib().wtg_fm_count(self.tree.h, _p(self.C), self.sigma, _p(pat) if pat.size else None, _p(off),
                               out.size, _p(out)))
        return out

    def count_device(self, d_C, d_pat, d_off, npat, d_out, stream=0):
        _ck(lib().wtg_fm_count_device(self.tree.h, vp(d_C), self.sigma, vp(d_pat), vp(d_off), npat, vp(d_out),
                                      vp(stream)))


class HuffmanTree:
    """Huffman-shaped wavelet tree of a byte text (sdsl::wt_huff<>) built on
    the GPU, with rank_support_v / select_support_mcl over its bitvector
    (include/wtg.h: wtg_huff_build)."""

    def __init__(self, text=None, flags=ALL, _handle=None):
        self.h = vp()
        if _handle is not None:
            self.h = _handle
        else:
            text = np.ascontiguousarray(text, dtype=np.uint8)
            _ck(lib().wtg_huff_build(_p(text), text.size, flags, ctypes.byref(self.h)))
        info = np.zeros(5, dtype=np.uint64)
        _ck(lib().wtg_huff_info(self.h, _p(info)))
        self.n, self.sigma, self.size, self.num_nodes, self.rank_words = [int(x) for x in info]

    @classmethod
    def from_device(cls, d_text, n, flags=ALL, stream=0):
        h = vp()
        _ck(lib().wtg_huff_build_device(vp(d_text), int(n), flags, vp(stream), ctypes.byref(h)))
        return cls(_handle=h)

    def free(self):
        if self.h:
            lib().wtg_huff_free(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def bits(self):
        out = np.zeros((self.size + 63) // 64, dtype=np.uint64)
        _ck(lib().wtg_huff_get_bits(self.h, _p(out), out.size))
        return out

    def tree(self):
        """(nodes [m, 5]: bv_pos, bv_pos_rank, parent, child0, child1; leaf
        per byte; path per byte, length in the top 8 bits)."""
        nodes = np.zeros((max(self.num_nodes, 1), 5), dtype=np.uint64)
        leaves, paths = np.zeros(256, dtype=np.uint64), np.zeros(256, dtype=np.uint64)
        _ck(lib().wtg_huff_get_tree(self.h, _p(nodes), _p(leaves), _p(paths)))
        return nodes[: self.num_nodes], leaves, paths

    def rank_table(self):
        out = np.zeros(self.rank_words, dtype=np.uint64)
        _ck(lib().wtg_huff_get_rank(self.h, _p(out), out.size))
        return out

    def select_tables(self, t_b):
        info = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_huff_select_info(self.h, t_b, _p(info)))
        sb = np.zeros(max(int(info[6]), 1), dtype=np.uint64)
        desc = np.zeros(max(int(info[4]), 1), dtype=np.uint64)
        pool = np.zeros(max(int(info[7]), 1), dtype=np.uint64)
        _ck(lib().wtg_huff_get_select(self.h, t_b, _p(sb), _p(desc), _p(pool)))
        return _SelectTables(info, sb[: int(info[6])], desc[: int(info[4])], pool[: int(info[7])])

    def access(self, idx):
        idx = _u64(idx)
        out = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_huff_access(self.h, _p(idx), idx.size, _p(out)))
        return out

    def rank(self, idx, sym):
        idx, sym = _u64(idx), _u64(sym)
        out = np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_huff_rank(self.h, _p(idx), _p(sym), idx.size, _p(out)))
        return out

    def select(self, i, sym):
        i, sym = _u64(i), _u64(sym)
        out = np.zeros(i.size, dtype=np.uint64)
        _ck(lib().wtg_huff_select(self.h, _p(i), _p(sym), i.size, _p(out)))
        return out

    def inverse_select(self, idx):
        idx = _u64(idx)
        r, c = np.zeros(idx.size, dtype=np.uint64), np.zeros(idx.size, dtype=np.uint64)
        _ck(lib().wtg_huff_inverse_select(self.h, _p(idx), idx.size, _p(r), _p(c)))
        return r, c

    def fm_count(self, C, pat, off):
        """Backward-search counts over the tree of a BWT: C[c] = bytes below c
        (256 entries), patterns pat[off[q]:off[q+1]] (bytes)."""
        C, off = _u64(C), _u64(off)
        pat = np.ascontiguousarray(pat, dtype=np.uint8)
        out = np.zeros(off.size - 1, dtype=np.uint64)
        _ck(lib().wtg_huff_fm_count(self.h, _p(C), _p(pat) if pat.size else None, _p(off), out.size, _p(out)))
        return out

    def fm_count_device(self, d_C, d_pat, d_off, npat, d_out, stream=0):
        """fm_count on device arrays (256 u64 C, u8 patterns, npat + 1 u64
        offsets, npat u64 counts), enqueued on `stream`."""
        _ck(lib().wtg_huff_fm_count_device(self.h, vp(d_C), vp(d_pat), vp(d_off), int(npat), vp(d_out), vp(stream)))


class Batch:
    """Many independent texts (u8 symbols, 1..4 levels), each with its own
    wavelet tree, rank_support_v and select_support_mcl, built in one
    persistent launch (include/wtg.h: wtg_batch_plan)."""

    def __init__(self, lengths, levels, flags=ALL, stream=0):
        self.h = vp()
        self.lengths = _u64(lengths)
        self.levels = int(levels)
        _ck(lib().wtg_batch_plan(_p(self.lengths), self.lengths.size, self.levels, flags, vp(stream),
                                 ctypes.byref(self.h)))

    @classmethod
    def from_texts(cls, texts, levels, flags=ALL):
        b = cls([len(t) for t in texts], levels, flags)
        b.load(np.concatenate([np.asarray(t, dtype=np.uint8) for t in texts]) if texts else np.zeros(0, np.uint8))
        return b

    def input_device(self):
        p, nb = vp(), ctypes.c_uint64(0)
        _ck(lib().wtg_batch_input(self.h, ctypes.byref(p), ctypes.byref(nb)))
        return p.value or 0, nb.value

    def load(self, concat):
        concat = np.ascontiguousarray(concat, dtype=np.uint8)
        _ck(lib().wtg_batch_load(self.h, _p(concat)))

    def run(self):
        _ck(lib().wtg_batch_run(self.h))

    def set_shape(self, tile=65536, whole_max=-1, symbols_per_thread=32):
        """Fix the shape instead of tuning it on the first run: symbols per
        split-text tile, the longest text one CTA builds whole (-1 automatic,
        0 split all), and the level pass's symbols per thread (32 or 64)."""
        _ck(lib().wtg_batch_set_shape(self.h, tile, whole_max, symbols_per_thread))

    def sync(self):
        _ck(lib().wtg_batch_sync(self.h))

    def free(self):
        if self.h:
            lib().wtg_batch_free(self.h)
            self.h = vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def text_info(self, t):
        a = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_batch_text_info(self.h, t, _p(a)))
        return dict(zip(("n", "levels", "bit_words", "rank_words", "ones", "zeros", "tile", "whole"),
                        (int(x) for x in a)))

    def bits(self, t):
        out = np.zeros(self.text_info(t)["bit_words"], dtype=np.uint64)
        _ck(lib().wtg_batch_get_bits(self.h, t, _p(out), out.size))
        return out

    def rank_table(self, t):
        out = np.zeros(self.text_info(t)["rank_words"], dtype=np.uint64)
        _ck(lib().wtg_batch_get_rank(self.h, t, _p(out), out.size))
        return out

    def select_tables(self, t, t_b):
        info = np.zeros(8, dtype=np.uint64)
        _ck(lib().wtg_batch_select_info(self.h, t, t_b, _p(info)))
        sb = np.zeros(max(int(info[6]), 1), dtype=np.uint64)
        desc = np.zeros(max(int(info[4]), 1), dtype=np.uint64)
        pool = np.zeros(max(int(info[7]), 1), dtype=np.uint64)
        _ck(lib().wtg_batch_get_select(self.h, t, t_b, _p(sb), _p(desc), _p(pool)))
        return _SelectTables(info, sb[: int(info[6])], desc[: int(info[4])], pool[: int(info[7])])

    def shape(self):
        """After a run: (split tile, whole-text bound in use, symbols per
        thread, texts built whole, candidate times in ms)."""
        th, wm, spt, nw = ctypes.c_int(0), ctypes.c_int64(0), ctypes.c_int(0), ctypes.c_uint64(0)
        ms = np.zeros(8, dtype=np.float32)
        _ck(lib().wtg_batch_shape(self.h, ctypes.byref(th), ctypes.byref(wm), ctypes.byref(spt), ctypes.byref(nw),
                                  _p(ms)))
        return th.value, wm.value, spt.value, nw.value, ms


def rank_build_noalloc(d_words_ptr, size_bits, d_rank_ptr, stream=0):
    """rank_support_v<1> table of a device bitvector into a device buffer,
    without any device allocation (include/wtg.h: wtg_rank_build_noalloc)."""
    _ck(lib().wtg_rank_build_noalloc(vp(d_words_ptr), int(size_bits), vp(d_rank_ptr), vp(stream)))


def rank_words(size_bits):
    """Words of a rank_support_v<1> table over size_bits bits."""
    if size_bits == 0:
        return 2
    cap = (size_bits + 63) // 64 * 64
    return ((cap >> 9) + 1) << 1


def remap_alphabet(seq):
    """levelWT/WTTime.C:80-94 on the GPU: returns (remapped copy, sigma)."""
    s = np.array(seq, copy=True)
    sigma = ctypes.c_uint64(0)
    _ck(lib().wtg_remap_alphabet(_p(s), s.size, s.dtype.itemsize, ctypes.byref(sigma)))
    return s, int(sigma.value)
