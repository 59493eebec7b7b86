"""ctypes binding of the CPU oracle (oracle/wt_oracle.c) and of the
reference-built WT() libraries (oracle/_ref/).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke entry and by the
benchmark's CPU-baseline leg, always as the checker or the timed CPU
baseline -- never as the product path.
"""
import ctypes
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# The reference checkout: $WTG_REFERENCE_DIR, else "reference" beside the repo root.
REF_SRC = os.environ.get("WTG_REFERENCE_DIR") or os.path.abspath(os.path.join(HERE, "..", "..", "reference"))

u64 = ctypes.c_uint64
vp = ctypes.c_void_p
NONE = np.uint64(0xFFFFFFFFFFFFFFFF)


def build(ref=True):
    """Compile the oracle; with ref=True also the reference's own builders:
    the pins (_ref/libref_*.so, where the reference checkout exists) and the
    timed CPU baseline (_ref/libref_bench_*.so, from the staged copy of the
    reference's sources in _ref/src, which also builds where the checkout
    does not exist)."""
    import shutil
    if shutil.which("make"):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
        if ref and os.path.isdir(REF_SRC):
            subprocess.run(["make", "-s", "-C", HERE, "ref", "ref-src", "REF=" + REF_SRC], check=True)
        if ref and os.path.isdir(os.path.join(REF_DIR, "src")):
            subprocess.run(["make", "-s", "-C", HERE, "bench-ref"], check=True)
        return
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    subprocess.run(["gcc", "-O2", "-fPIC", "-fopenmp", "-std=gnu11", "-shared", "-o", LIB_PATH,
                    os.path.join(HERE, "wt_oracle.c")], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.or_log2_up.argtypes = [u64]
        L.or_hi.argtypes = [u64]
        L.or_levels_for_sigma.argtypes = [u64]
        L.or_wt_levelwt.argtypes = [vp, ctypes.c_int, u64, ctypes.c_int, vp, vp, u64]
        L.or_wt_serial.argtypes = [vp, ctypes.c_int, u64, ctypes.c_int, vp, vp, u64]
        L.or_remap_alphabet.argtypes = [vp, ctypes.c_int, u64]
        L.or_remap_alphabet.restype = u64
        L.or_rank_words.argtypes = [u64]
        L.or_rank_words.restype = u64
        L.or_rank_build.argtypes = [vp, u64, vp]
        L.or_rank1.argtypes = [vp, vp, u64]
        L.or_rank1.restype = u64
        L.or_select_new.argtypes = [vp, u64, ctypes.c_int, ctypes.c_int]
        L.or_select_new.restype = vp
        L.or_select_info.argtypes = [vp, vp]
        L.or_select_copy.argtypes = [vp, vp, vp, vp]
        L.or_select_query.argtypes = [vp, vp, u64]
        L.or_select_query.restype = u64
        L.or_select_batch.argtypes = [vp, vp, vp, u64, vp]
        L.or_select_free.argtypes = [vp]
        L.or_wt_access.argtypes = [vp, vp, u64, ctypes.c_int, u64]
        L.or_wt_access.restype = u64
        L.or_wt_rank.argtypes = [vp, vp, u64, ctypes.c_int, u64, u64]
        L.or_wt_rank.restype = u64
        L.or_wt_inverse_select.argtypes = [vp, vp, u64, ctypes.c_int, u64, vp]
        L.or_wt_inverse_select.restype = u64
        L.or_wt_select.argtypes = [vp, vp, vp, vp, u64, ctypes.c_int, u64, u64]
        L.or_wt_select.restype = u64
        L.or_wt_access_batch.argtypes = [vp, vp, u64, ctypes.c_int, vp, u64, vp]
        L.or_wt_rank_batch.argtypes = [vp, vp, u64, ctypes.c_int, vp, vp, u64, vp]
        ci = ctypes.c_int
        L.or_wt_lex_count.argtypes = [vp, vp, u64, ci, u64, u64, u64, vp]
        L.or_wt_lex_smaller_count.argtypes = [vp, vp, u64, ci, u64, u64, vp]
        L.or_wt_range_search_2d.argtypes = [vp, vp, vp, vp, u64, ci, u64, u64, u64, u64, ci, u64, vp, vp]
        L.or_wt_range_search_2d.restype = u64
        L.or_wt_interval_symbols.argtypes = [vp, vp, u64, ci, u64, u64, u64, vp, vp, vp]
        L.or_wt_interval_symbols.restype = u64
        L.or_wt_expand.argtypes = [vp, vp, u64, vp, vp, vp]
        L.or_wt_expand_ranges.argtypes = [vp, vp, vp, vp, u64, vp, vp]
        L.or_wt_lex_count_batch.argtypes = [vp, vp, u64, ci, vp, vp, vp, u64, vp]
        L.or_wt_lex_smaller_count_batch.argtypes = [vp, vp, u64, ci, vp, vp, u64, vp]
        L.or_wt_range_count_batch.argtypes = [vp, vp, u64, ci, vp, vp, vp, vp, u64, vp]
        L.or_num_threads.restype = ctypes.c_int
        L.or_suffix_array_u8.argtypes = [vp, ctypes.c_int64, vp]
        L.or_suffix_array_u8.restype = ctypes.c_int
        L.or_bwt_u8.argtypes = [vp, vp, ctypes.c_int64, vp]
        L.or_fm_count.argtypes = [vp, vp, u64, ctypes.c_int, vp, u64, vp, vp, u64, vp]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def num_threads():
    return lib().or_num_threads()


def levels_for_sigma(sigma):
    return lib().or_levels_for_sigma(int(sigma))


def log2_up(x):
    return lib().or_log2_up(int(x))


def hi(x):
    return lib().or_hi(int(x))


def wt_words(n, levels):
    return (n * levels + 63) // 64


def wt_build(sym, levels, n_nodes=None, serial=False, tail=False):
    """levelWT (or serialWT) build. Returns (words u64[], nodes u64[n_nodes,5] or None).
    With tail=True the words carry one extra zero word (the padding word
    rank_support_v reads past a bitvector whose size is a multiple of 512)."""
    sym = np.ascontiguousarray(sym)
    n = sym.size
    words = np.zeros(max(wt_words(n, levels), 1) + (1 if tail else 0), dtype=np.uint64)
    nodes = None
    if n_nodes:
        nodes = np.zeros((n_nodes, 5), dtype=np.uint64)
    fn = lib().or_wt_serial if serial else lib().or_wt_levelwt
    rc = fn(_p(sym), sym.dtype.itemsize, n, levels, _p(words), _p(nodes), n_nodes or 0)
    if rc != 0:
        raise RuntimeError(f"oracle wt build failed rc={rc}")
    return words[: wt_words(n, levels) + (1 if tail else 0)], nodes


def remap_alphabet(sym):
    s = np.array(sym, copy=True)
    sigma = lib().or_remap_alphabet(_p(s), s.dtype.itemsize, s.size)
    return s, int(sigma)


def rank_build(words, size_bits):
    words = np.ascontiguousarray(words, dtype=np.uint64)
    tbl = np.zeros(lib().or_rank_words(size_bits), dtype=np.uint64)
    lib().or_rank_build(_p(words), size_bits, _p(tbl))
    return tbl


def rank1(tbl, words, idx):
    return lib().or_rank1(_p(tbl), _p(words), int(idx))


class Select:
    """select_support_mcl<t_b> built by the oracle, in the flat packed layout."""

    def __init__(self, words, size_bits, t_b, rule=0):
        self.words = np.ascontiguousarray(words, dtype=np.uint64)
        self.h = lib().or_select_new(_p(self.words), size_bits, t_b, rule)
        info = np.zeros(8, dtype=np.uint64)
        lib().or_select_info(self.h, _p(info))
        (self.size, self.arg_cnt, self.logn, self.logn4, self.nsb, self.has_long,
         self.sb_nwords, self.pool_nwords) = [int(x) for x in info]
        self.sb_words = np.zeros(max(self.sb_nwords, 1), dtype=np.uint64)
        self.desc = np.zeros(max(self.nsb, 1), dtype=np.uint64)
        self.pool = np.zeros(max(self.pool_nwords, 1), dtype=np.uint64)
        lib().or_select_copy(self.h, _p(self.sb_words), _p(self.desc), _p(self.pool))
        self.sb_words = self.sb_words[: self.sb_nwords]
        self.desc = self.desc[: self.nsb]
        self.pool = self.pool[: self.pool_nwords]

    def query(self, i):
        return lib().or_select_query(self.h, _p(self.words), int(i))

    def query_batch(self, q):
        q = np.ascontiguousarray(q, dtype=np.uint64)
        out = np.zeros(q.size, dtype=np.uint64)
        lib().or_select_batch(self.h, _p(self.words), _p(q), q.size, _p(out))
        return out

    def __del__(self):
        try:
            if self.h:
                lib().or_select_free(self.h)
                self.h = None
        except Exception:
            pass


def wt_access(tree, rtbl, n, levels, idx):
    idx = np.ascontiguousarray(idx, dtype=np.uint64)
    out = np.zeros(idx.size, dtype=np.uint64)
    lib().or_wt_access_batch(_p(tree), _p(rtbl), n, levels, _p(idx), idx.size, _p(out))
    return out


def wt_rank(tree, rtbl, n, levels, idx, sym):
    idx = np.ascontiguousarray(idx, dtype=np.uint64)
    sym = np.ascontiguousarray(sym, dtype=np.uint64)
    out = np.zeros(idx.size, dtype=np.uint64)
    lib().or_wt_rank_batch(_p(tree), _p(rtbl), n, levels, _p(idx), _p(sym), idx.size, _p(out))
    return out


def wt_inverse_select(tree, rtbl, n, levels, i):
    c = ctypes.c_uint64(0)
    r = lib().or_wt_inverse_select(_p(tree), _p(rtbl), n, levels, int(i), ctypes.byref(c))
    return int(r), int(c.value)


def wt_select(tree, rtbl, sel1, sel0, n, levels, i, c):
    return lib().or_wt_select(_p(tree), _p(rtbl), ctypes.c_void_p(sel1.h), ctypes.c_void_p(sel0.h),
                              n, levels, int(i), int(c))


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def wt_lex_count(tree, rtbl, n, levels, i, j, c):
    """wt_int::lex_count per query: rows (rank(i, c), smaller, greater)."""
    i, j, c = _u64(i), _u64(j), _u64(c)
    out = np.zeros((i.size, 3), dtype=np.uint64)
    lib().or_wt_lex_count_batch(_p(tree), _p(rtbl), n, levels, _p(i), _p(j), _p(c), i.size, _p(out))
    return out


def wt_lex_smaller_count(tree, rtbl, n, levels, i, c):
    """wt_int::lex_smaller_count per query: rows (rank(i, c), smaller)."""
    i, c = _u64(i), _u64(c)
    out = np.zeros((i.size, 2), dtype=np.uint64)
    lib().or_wt_lex_smaller_count_batch(_p(tree), _p(rtbl), n, levels, _p(i), _p(c), i.size, _p(out))
    return out


def wt_range_count(tree, rtbl, n, levels, lb, rb, vlb, vrb):
    """range_search_2d(lb, rb, vlb, vrb, report=false).first per query."""
    lb, rb, vlb, vrb = _u64(lb), _u64(rb), _u64(vlb), _u64(vrb)
    out = np.zeros(lb.size, dtype=np.uint64)
    lib().or_wt_range_count_batch(_p(tree), _p(rtbl), n, levels, _p(lb), _p(rb), _p(vlb), _p(vrb), lb.size,
                                  _p(out))
    return out


def wt_range_report(tree, rtbl, sel1, sel0, n, levels, lb, rb, vlb, vrb):
    """range_search_2d(lb, rb, vlb, vrb) of one query: (positions, values)."""
    cnt = lib().or_wt_range_search_2d(_p(tree), _p(rtbl), None, None, n, levels, int(lb), int(rb), int(vlb),
                                      int(vrb), 0, 0, None, None)
    pos = np.zeros(max(cnt, 1), dtype=np.uint64)
    val = np.zeros(max(cnt, 1), dtype=np.uint64)
    lib().or_wt_range_search_2d(_p(tree), _p(rtbl), ctypes.c_void_p(sel1.h), ctypes.c_void_p(sel0.h), n,
                                levels, int(lb), int(rb), int(vlb), int(vrb), 1, cnt, _p(pos), _p(val))
    return pos[:cnt], val[:cnt]


def wt_interval_symbols(tree, rtbl, n, levels, i, j):
    """interval_symbols(i, j) of one query: (symbols, rank(i, c), rank(j, c))."""
    cap = min(1 << levels, max(int(j) - int(i), 1)) if int(j) >= int(i) else 1
    cs, ri, rj = (np.zeros(cap, dtype=np.uint64) for _ in range(3))
    k = lib().or_wt_interval_symbols(_p(tree), _p(rtbl), n, levels, int(i), int(j), cap, _p(cs), _p(ri), _p(rj))
    return cs[:k], ri[:k], rj[:k]


def wt_expand(tree, rtbl, n, node):
    """expand(v): the children (offset, size, level, sym) of node v."""
    v = _u64(node)
    left, right = np.zeros(4, dtype=np.uint64), np.zeros(4, dtype=np.uint64)
    lib().or_wt_expand(_p(tree), _p(rtbl), n, _p(v), _p(left), _p(right))
    return left, right


def wt_expand_ranges(tree, rtbl, node, ranges):
    """expand(v, ranges): closed ranges [s, e] (rows) mapped to v's children."""
    v, r = _u64(node), _u64(ranges).reshape(-1, 2)
    left, right = np.zeros_like(r), np.zeros_like(r)
    lib().or_wt_expand_ranges(_p(tree), _p(rtbl), _p(v), _p(r), r.shape[0], _p(left), _p(right))
    return left, right


# ------------------------------------------------------ sdsl serialize()
# The byte streams of sdsl's serialize(), restated from the reference's
# members (wt_int/wt_int_par.hpp:887-899, rank/rank_support_v_par.hpp:154-164,
# select/select_support_mcl_par.hpp:644-681) and sdsl's int_vector format:
# size in bits (u64), width (u8, run-time widths only), ceil(bits/64) words.


def _iv(bits, words, width=None):
    head = struct.pack("<Q", int(bits)) + (b"" if width is None else struct.pack("<B", int(width)))
    w = np.ascontiguousarray(words, dtype="<u8")[: (int(bits) + 63) // 64]
    return head + w.tobytes()


def serialize_rank(tbl):
    """rank_support_v<1>::serialize: m_basic_block as an int_vector<64>."""
    return np.frombuffer(_iv(np.asarray(tbl).size * 64, tbl), dtype=np.uint8)


def serialize_select(sel):
    """select_support_mcl<t_b>::serialize of a Select (or RefSelect) built here."""
    out = [struct.pack("<Q", sel.arg_cnt)]
    if sel.arg_cnt:
        nsb = sel.nsb
        out.append(_iv(nsb * sel.logn, sel.sb_words, sel.logn))
        desc = np.asarray(sel.desc, dtype=np.uint64)
        if sel.has_long:
            mini = np.zeros((nsb + 63) // 64 * 64, dtype=bool)
            mini[:nsb] = ((desc >> np.uint64(7)) & np.uint64(1)) == 0
            out.append(_iv(nsb, np.packbits(mini, bitorder="little").view(np.uint64)))
        else:
            out.append(_iv(0, np.zeros(0, np.uint64)))
        pool = np.asarray(sel.pool, dtype=np.uint64)
        for d in desc.tolist():
            w, at = d & 0x7F, d >> 8
            entries = 4096 if (d >> 7) & 1 else 64
            out.append(_iv(entries * w, pool[at: at + entries * w // 64], w))
    return np.frombuffer(b"".join(out), dtype=np.uint8)


def serialize_wt_int(sym, levels):
    """wt_int<>(sym, n, levels)::serialize, built with this oracle."""
    sym = np.ascontiguousarray(sym)
    n = sym.size
    if n == 0:  # the constructor returns before building anything
        b = struct.pack("<QQ", 0, 0) + _iv(0, []) + _iv(0, []) + struct.pack("<QQI", 0, 0, 0)
        return np.frombuffer(b, dtype=np.uint8)
    w, _ = wt_build(sym, levels, tail=True)
    size = n * levels
    mask = (1 << levels) - 1
    sigma = np.unique(sym.astype(np.uint64) & np.uint64(mask)).size
    parts = [struct.pack("<QQ", n, sigma), _iv(size, w),
             serialize_rank(rank_build(w, size)).tobytes(),
             serialize_select(Select(w, size, 1)).tobytes(), serialize_select(Select(w, size, 0)).tobytes(),
             struct.pack("<I", levels)]
    return np.frombuffer(b"".join(parts), dtype=np.uint8)


# ------------------------------------------------- Huffman-shaped tree
# Restates the reference's wt_huff build (wt_huff/wt_huff_par.hpp:82-117 for
# the shape, wt_huff/wt_pc_par.hpp:193-258,321-361 for the bits) over the
# breadth-first byte code tree of sdsl's byte_tree.


class HuffShape:
    """The code tree of a byte text: nodes in breadth-first order (root 0) as
    rows (bv_pos, freq, sym, parent, child0, child1) -- -1 for no parent /
    child -- and per byte its path (bit d set: the (d+1)-th edge goes right)
    and path length (0: not in the text).  bv_size = the concatenated
    bitvector's length (the inner nodes' sizes)."""

    def __init__(self, counts):
        import heapq
        counts = [int(c) for c in counts]
        shape = []  # [freq, sym, child0, child1]
        heap = []
        for c, f in enumerate(counts):
            if f > 0:
                heap.append((f, len(shape)))
                shape.append([f, c, -1, -1])
        heapq.heapify(heap)
        while len(heap) > 1:  # the two smallest (frequency, node number) pairs merge
            f1, i1 = heapq.heappop(heap)
            f2, i2 = heapq.heappop(heap)
            heapq.heappush(heap, (f1 + f2, len(shape)))
            shape.append([f1 + f2, 0, i1, i2])
        rows, order = [], []
        if shape:
            order = [len(shape) - 1]
            rows = [[0, 0, 0, -1, -1, -1]]
        bv = 0
        k = 0
        while k < len(order):  # first in, first out: the placed nodes are the queue
            f, sym, c0, c1 = shape[order[k]]
            rows[k][0], rows[k][1], rows[k][2] = bv, f, sym
            if c0 >= 0:
                bv += f
                for j, c in enumerate((c0, c1)):
                    rows[k][4 + j] = len(order)
                    order.append(c)
                    rows.append([0, 0, 0, k, -1, -1])
            k += 1
        self.nodes = np.array(rows, dtype=np.int64).reshape(-1, 6)
        self.bv_size = bv
        self.sigma = sum(1 for f in counts if f > 0)
        self.leaf = np.full(256, -1, dtype=np.int64)
        self.path = np.zeros(256, dtype=np.uint64)
        self.plen = np.zeros(256, dtype=np.int64)
        for v in range(self.nodes.shape[0]):
            if self.nodes[v, 4] < 0:
                c = int(self.nodes[v, 2])
                self.leaf[c] = v
                p, ln, u = 0, 0, v
                while u != 0:
                    par = int(self.nodes[u, 3])
                    p = (p << 1) | (1 if int(self.nodes[par, 5]) == u else 0)
                    ln += 1
                    u = par
                self.path[c], self.plen[c] = p, ln


def huff_build(text):
    """wt_huff over a byte text: (HuffShape, words of the concatenated
    bitvector with one zero word after the data)."""
    text = np.ascontiguousarray(text, dtype=np.uint8)
    counts = np.bincount(text, minlength=256) if text.size else np.zeros(256, np.int64)
    sh = HuffShape(counts[: int(text.max()) + 1] if text.size else [])
    nwords = (sh.bv_size + 63) // 64
    words = np.zeros(nwords + 1, dtype=np.uint64)
    if text.size == 0 or sh.bv_size == 0:
        return sh, words
    plen = sh.plen[text]
    path = sh.path[text]
    bits = np.zeros(sh.bv_size, dtype=np.uint8)
    # depth d: the symbols whose code is longer than d, stably ordered by the
    # depth-d node on their path (breadth-first = left to right), give the
    # bits of the depth-d inner nodes, which lie consecutively from the first
    # one's bv_pos
    node = np.zeros(text.size, dtype=np.int64)  # each symbol's node at depth d
    for d in range(int(plen.max())):
        live = plen > d
        idx = np.nonzero(live)[0]
        if idx.size == 0:
            break
        nd = node[idx]
        o = np.argsort(sh.nodes[nd, 0], kind="stable")
        b = ((path[idx] >> np.uint64(d)) & np.uint64(1)).astype(np.int64)
        start = int(sh.nodes[nd[o[0]], 0])
        bits[start:start + idx.size] = b[o]
        node[idx] = sh.nodes[nd, 4 + b]
    words[:nwords] = np.packbits(np.concatenate([bits, np.zeros(nwords * 64 - bits.size, np.uint8)]),
                                 bitorder="little").view(np.uint64)
    return sh, words


class HuffOracle:
    """wt_huff built here, with rank_support_v / select_support_mcl over its
    bitvector and the wt_pc queries (wt_huff/wt_pc_par.hpp:430-552)."""

    def __init__(self, text):
        self.text = np.ascontiguousarray(text, dtype=np.uint8)
        self.n = self.text.size
        self.shape, self.words = huff_build(self.text)
        self.size = self.shape.bv_size
        self.rank_tbl = rank_build(self.words, self.size)
        nd = self.shape.nodes
        self.node_rank = np.array([rank1(self.rank_tbl, self.words, int(nd[v, 0])) if nd[v, 4] >= 0 else int(nd[v, 2])
                                   for v in range(nd.shape[0])], dtype=np.uint64)
        self.sel = {t_b: Select(self.words, self.size, t_b) for t_b in (0, 1)}

    def _bit(self, p):
        return (int(self.words[p >> 6]) >> (p & 63)) & 1

    def _r1(self, p):
        return rank1(self.rank_tbl, self.words, p)

    def access(self, i):
        nd, v = self.shape.nodes, 0
        while nd[v, 4] >= 0:
            p = int(nd[v, 0]) + i
            r = self._r1(p) - int(self.node_rank[v])
            if self._bit(p):
                i, v = r, int(nd[v, 5])
            else:
                i, v = i - r, int(nd[v, 4])
        return int(nd[v, 2])

    def rank(self, i, c):
        sh, nd = self.shape, self.shape.nodes
        if sh.leaf[c] < 0:
            return 0
        if sh.sigma == 1:
            return i
        p, ln, res, v = int(sh.path[c]), int(sh.plen[c]), i, 0
        for _ in range(ln):
            if res == 0:
                break
            r = self._r1(int(nd[v, 0]) + res) - int(self.node_rank[v])
            res = r if p & 1 else res - r
            v = int(nd[v, 5 if p & 1 else 4])
            p >>= 1
        return res

    def select(self, i, c):
        sh, nd = self.shape, self.shape.nodes
        v = int(sh.leaf[c])
        if v < 0:
            return self.n
        if sh.sigma == 1:
            return min(i - 1, self.n)
        res = i - 1
        for _ in range(int(sh.plen[c])):
            par = int(nd[v, 3])
            if int(nd[par, 5]) == v:
                res = self.sel[1].query(int(self.node_rank[par]) + res + 1) - int(nd[par, 0])
            else:
                res = self.sel[0].query(int(nd[par, 0]) - int(self.node_rank[par]) + res + 1) - int(nd[par, 0])
            v = par
        return res


# ---------------------------------------------------------------- reference

_ref_libs = {}


def suffix_array(s):
    """Suffix array of a byte string (no sentinel), int64."""
    s = np.ascontiguousarray(s, dtype=np.uint8)
    sa = np.zeros(s.size, dtype=np.int64)
    if lib().or_suffix_array_u8(_p(s), s.size, _p(sa)) != 0:
        raise MemoryError("oracle suffix array")
    return sa


def bwt(s, sa):
    """fm-index/par/WT.C:38-41: s[sa[i]-1], or s[n-1] where sa[i] == 0."""
    s = np.ascontiguousarray(s, dtype=np.uint8)
    sa = np.ascontiguousarray(sa, dtype=np.int64)
    out = np.zeros(s.size, dtype=np.uint8)
    lib().or_bwt_u8(_p(s), _p(sa), s.size, _p(out))
    return out


def fm_count(tree, rtbl, n, levels, C, pat, off):
    """Backward-search counts of the patterns pat[off[p]:off[p+1]] (codes);
    C[c] = codes below c, one entry per code."""
    C = np.ascontiguousarray(C, dtype=np.uint64)
    pat = np.ascontiguousarray(pat, dtype=np.uint8)
    off = np.ascontiguousarray(off, dtype=np.uint64)
    out = np.zeros(off.size - 1, dtype=np.uint64)
    lib().or_fm_count(_p(tree), _p(rtbl), n, levels, _p(C), C.size, _p(pat) if pat.size else None,
                      _p(off), out.size, _p(out))
    return out


def ref_divsufsort(s):
    """The reference's vendored divsufsort (suffixArray/divsufsort), int32 SA."""
    L = ctypes.CDLL(os.path.join(REF_DIR, "libref_divsufsort.so"))
    L.divsufsort.argtypes = [vp, vp, ctypes.c_int32]
    L.divsufsort.restype = ctypes.c_int32
    s = np.ascontiguousarray(s, dtype=np.uint8)
    sa = np.zeros(max(s.size, 1), dtype=np.int32)
    if L.divsufsort(_p(s), _p(sa), s.size) != 0:
        raise RuntimeError("divsufsort failed")
    return sa[: s.size]


_ref_bench = None


def ref_bench():
    """The reference's own CPU builders compiled for the timed baseline
    (levelWT with -DLONG -DINT and with byte symbols, rank_support_v_par and
    select_support_mcl_par, all with OpenMP) as (wt_long_int, rs, wt_u8), or
    None where they were not built."""
    global _ref_bench
    if _ref_bench is None:
        paths = [os.path.join(REF_DIR, f"libref_bench_{v}.so") for v in ("levelwt", "rs", "levelwt_u8")]
        if not all(os.path.exists(p) for p in paths):
            return None
        wt, rs, wt8 = (ctypes.CDLL(p) for p in paths)
        for w in (wt, wt8):
            w.ref_wt_time.argtypes = [vp, ctypes.c_int, u64, u64]
            w.ref_wt_time.restype = ctypes.c_double
            w.ref_wt_batch_time.argtypes = [vp, vp, u64, u64]
            w.ref_wt_batch_time.restype = ctypes.c_double
        rs.ref_rank_select_time.argtypes = [vp, u64, vp]
        rs.ref_rank_select_batch_time.argtypes = [vp, vp, vp, u64]
        rs.ref_rank_select_batch_time.restype = ctypes.c_double
        rs.ref_select_new.argtypes = [vp, u64, ctypes.c_int]
        rs.ref_select_new.restype = vp
        rs.ref_select_free.argtypes = [vp]
        rs.ref_select_batch.argtypes = [vp, vp, u64, vp]
        rs.ref_select_batch.restype = ctypes.c_double
        _ref_bench = (wt, rs, wt8)
    return _ref_bench


def ref_bench_byte_text(sym, levels):
    """Seconds of the reference's WT() over a byte text (sigma 2^levels) and
    of its rank_support_v constructor over those bits: (t_wt, t_rank)."""
    wt, rs, wt8 = ref_bench()
    sym = np.ascontiguousarray(sym, dtype=np.uint8)
    t_wt = wt8.ref_wt_time(_p(sym), 1, sym.size, 1 << levels)
    w, _ = wt_build(sym, levels, tail=True)
    out = np.zeros(5)
    rs.ref_rank_select_time(_p(w), sym.size * levels, _p(out))
    return t_wt, float(out[0])


def ref_bench_batch(concat, lengths, levels):
    """Seconds of the reference's WT() per text and of its rank_support_v +
    select_support_mcl<1> + <0> per text, the texts spread over the OpenMP
    threads: (t_wt, t_supports)."""
    wt, rs, wt8 = ref_bench()
    concat = np.ascontiguousarray(concat, dtype=np.uint8)
    lengths = np.asarray(lengths, dtype=np.uint64)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)
    t_wt = wt8.ref_wt_batch_time(_p(concat), _p(offs), lengths.size, 1 << levels)
    words, woffs, sizes = [], [0], []
    for t in range(lengths.size):
        w, _ = wt_build(concat[int(offs[t]):int(offs[t + 1])], levels, tail=True)
        words.append(w)
        woffs.append(woffs[-1] + w.size)
        sizes.append(int(lengths[t]) * levels)
    allw = np.concatenate(words) if words else np.zeros(1, np.uint64)
    wo = np.asarray(woffs[:-1], dtype=np.uint64)  # kept alive across the call
    sz = np.asarray(sizes, dtype=np.uint64)
    t_rs = rs.ref_rank_select_batch_time(_p(allw), _p(wo), _p(sz), lengths.size)
    return t_wt, t_rs


def ref_bench_select(words, size_bits, t_b, queries):
    """The reference's select_support_mcl<t_b>::select over a bitvector for
    every query (OpenMP over the queries): (seconds, answers)."""
    wt, rs, wt8 = ref_bench()
    words = np.ascontiguousarray(words, dtype=np.uint64)
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    out = np.zeros(q.size, dtype=np.uint64)
    h = rs.ref_select_new(_p(words), size_bits, t_b)
    try:
        secs = rs.ref_select_batch(h, _p(q), q.size, _p(out))
    finally:
        rs.ref_select_free(h)
    return secs, out


def ref_bench_times(sym, levels):
    """Seconds of the reference's WT(s, n, 2^levels), and of its
    rank_support_v / select_support_mcl<1> / <0> constructors over those
    bits, for one sample; plus the select structures' words (for the
    algorithmic bytes).  Returns (t_wt, t_rank, t_sel1, t_sel0, sel_words)."""
    wt, rs, _ = ref_bench()
    sym = np.ascontiguousarray(sym)
    t_wt = wt.ref_wt_time(_p(sym), sym.dtype.itemsize, sym.size, 1 << levels)
    if t_wt < 0:
        raise MemoryError("reference WT() sample")
    w, _ = wt_build(sym, levels, tail=True)  # the same bits (pinned), to feed the supports
    out = np.zeros(5)
    rs.ref_rank_select_time(_p(w), sym.size * levels, _p(out))
    return t_wt, out[0], out[1], out[2], int(out[3] + out[4])


def ref_available(variant="levelwt_u8"):
    return os.path.exists(os.path.join(REF_DIR, f"libref_{variant}.so"))


def ref_wt(sym, sigma, variant="levelwt_u8"):
    """The reference's own WT(s, n, sigma) (built from its sources into _ref/).
    Returns (words u64[], nodes as a structured u32/u64 array [2*sigma,5])."""
    if variant not in _ref_libs:
        L = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{variant}.so"))
        L.ref_wt.argtypes = [vp, u64, u64, vp, u64, vp]
        _ref_libs[variant] = L
    L = _ref_libs[variant]
    sb, ub = L.ref_symbol_bytes(), L.ref_uint_bytes()
    sym = np.ascontiguousarray(sym, dtype={1: np.uint8, 4: np.uint32, 8: np.uint64}[sb])
    n = sym.size
    levels = levels_for_sigma(sigma)
    nw = wt_words(n, levels)
    words = np.zeros(max(nw, 1), dtype=np.uint64)
    nodes = np.zeros((2 * sigma, 5), dtype=np.uint32 if ub == 4 else np.uint64)
    rc = L.ref_wt(_p(sym), n, sigma, _p(words), nw, _p(nodes))
    if rc != 0:
        raise RuntimeError("reference WT failed")
    return words[:nw], nodes


def reachable_nodes(nodes, none_value):
    """Heap ids reachable from the root through the child links."""
    seen = []
    stack = [0]
    while stack:
        h = stack.pop()
        seen.append(h)
        for c in (int(nodes[h, 3]), int(nodes[h, 4])):
            if c != int(none_value):
                stack.append(c)
    return sorted(seen)


_ref_rs = None


def _ref_rank_select():
    global _ref_rs
    if _ref_rs is None:
        L = ctypes.CDLL(os.path.join(REF_DIR, "libref_rank_select.so"))
        L.ref_rank_build.argtypes = [vp, u64, vp, u64]
        L.ref_rank_query.argtypes = [vp, u64, u64]
        L.ref_rank_query.restype = u64
        L.ref_select_new.argtypes = [vp, u64, ctypes.c_int]
        L.ref_select_new.restype = vp
        L.ref_select_info.argtypes = [vp, vp]
        L.ref_select_copy.argtypes = [vp, vp, vp, vp]
        L.ref_select_query.argtypes = [vp, u64]
        L.ref_select_query.restype = u64
        L.ref_select_free.argtypes = [vp]
        L.ref_rank_serialize.argtypes = [vp, u64, vp, u64]
        L.ref_rank_serialize.restype = u64
        L.ref_select_serialize.argtypes = [vp, vp, u64]
        L.ref_select_serialize.restype = u64
        _ref_rs = L
    return _ref_rs


def ref_rank_build(words, size_bits):
    """The reference's rank_support_v<1> table (m_basic_block)."""
    words = np.ascontiguousarray(words, dtype=np.uint64)
    tbl = np.zeros(lib().or_rank_words(size_bits), dtype=np.uint64)
    if _ref_rank_select().ref_rank_build(_p(words), size_bits, _p(tbl), tbl.size) != 0:
        raise RuntimeError("reference rank table size mismatch")
    return tbl


def ref_rank_serialize(words, size_bits):
    """The reference's rank_support_v<1>::serialize stream."""
    words = np.ascontiguousarray(words, dtype=np.uint64)
    L = _ref_rank_select()
    n = L.ref_rank_serialize(_p(words), size_bits, None, 0)
    out = np.zeros(n, dtype=np.uint8)
    L.ref_rank_serialize(_p(words), size_bits, _p(out), n)
    return out


class RefSelect:
    """The reference's select_support_mcl<t_b>, exported in the flat packed layout."""

    def __init__(self, words, size_bits, t_b):
        L = _ref_rank_select()
        self.words = np.ascontiguousarray(words, dtype=np.uint64)
        self.h = L.ref_select_new(_p(self.words), size_bits, t_b)
        info = np.zeros(8, dtype=np.uint64)
        L.ref_select_info(self.h, _p(info))
        (self.size, self.arg_cnt, self.logn, self.logn4, self.nsb, self.has_long,
         self.sb_nwords, self.pool_nwords) = [int(x) for x in info]
        self.sb_words = np.zeros(max(self.sb_nwords, 1), dtype=np.uint64)
        self.desc = np.zeros(max(self.nsb, 1), dtype=np.uint64)
        self.pool = np.zeros(max(self.pool_nwords, 1), dtype=np.uint64)
        L.ref_select_copy(self.h, _p(self.sb_words), _p(self.desc), _p(self.pool))
        self.sb_words = self.sb_words[: self.sb_nwords]
        self.desc = self.desc[: self.nsb]
        self.pool = self.pool[: self.pool_nwords]

    def query(self, i):
        return _ref_rank_select().ref_select_query(self.h, int(i))

    def serialize(self):
        """The reference's select_support_mcl::serialize stream."""
        L = _ref_rank_select()
        n = L.ref_select_serialize(self.h, None, 0)
        out = np.zeros(n, dtype=np.uint8)
        L.ref_select_serialize(self.h, _p(out), n)
        return out

    def __del__(self):
        try:
            if self.h:
                _ref_rank_select().ref_select_free(self.h)
                self.h = None
        except Exception:
            pass


_ref_wi = None


def _ref_wt_int():
    global _ref_wi
    if _ref_wi is None:
        L = ctypes.CDLL(os.path.join(REF_DIR, "libref_wt_int.so"))
        L.ref_wtint_new.argtypes = [vp, ctypes.c_int, u64, ctypes.c_uint32]
        L.ref_wtint_new.restype = vp
        L.ref_wtint_free.argtypes = [vp]
        L.ref_wtint_info.argtypes = [vp, vp]
        L.ref_wtint_bits.argtypes = [vp, vp]
        for f in ("ref_wtint_access",):
            getattr(L, f).argtypes = [vp, u64]
            getattr(L, f).restype = u64
        L.ref_wtint_rank.argtypes = [vp, u64, u64]
        L.ref_wtint_rank.restype = u64
        L.ref_wtint_select.argtypes = [vp, u64, u64]
        L.ref_wtint_select.restype = u64
        L.ref_wtint_inverse_select.argtypes = [vp, u64, vp]
        L.ref_wtint_lex_count.argtypes = [vp, u64, u64, u64, vp]
        L.ref_wtint_lex_smaller_count.argtypes = [vp, u64, u64, vp]
        L.ref_wtint_interval_symbols.argtypes = [vp, u64, u64, u64, vp, vp, vp]
        L.ref_wtint_interval_symbols.restype = u64
        L.ref_wtint_range_search_2d.argtypes = [vp, u64, u64, u64, u64, ctypes.c_int, u64, vp, vp]
        L.ref_wtint_range_search_2d.restype = u64
        L.ref_wtint_expand.argtypes = [vp, vp, vp, vp]
        L.ref_wtint_expand_ranges.argtypes = [vp, vp, vp, u64, vp, vp]
        L.ref_wtint_serialize.argtypes = [vp, vp, u64]
        L.ref_wtint_serialize.restype = u64
        L.ref_wtint_load.argtypes = [vp, u64]
        L.ref_wtint_load.restype = vp
        _ref_wi = L
    return _ref_wi


class RefWtHuff:
    """The reference's own wt_huff (wt_huff/wt_huff_par.hpp over
    wt_huff/wt_pc_par.hpp), built by its constructor and queried through its
    members; its tree in the shim's breadth-first node layout."""

    def __init__(self, text):
        L = ctypes.CDLL(os.path.join(REF_DIR, "libref_wt_huff.so"))
        L.ref_huff_new.argtypes = [vp, u64]
        L.ref_huff_new.restype = vp
        L.ref_huff_free.argtypes = [vp]
        for f in ("ref_huff_info", "ref_huff_bits", "ref_huff_rank"):
            getattr(L, f).argtypes = [vp, vp]
        L.ref_huff_rank_words.argtypes = [vp]
        L.ref_huff_rank_words.restype = u64
        L.ref_huff_nodes.argtypes = [vp, vp, vp, vp]
        L.ref_huff_select.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
        L.ref_huff_access.argtypes = [vp, u64]
        L.ref_huff_access.restype = u64
        L.ref_huff_rank_query.argtypes = [vp, u64, u64]
        L.ref_huff_rank_query.restype = u64
        L.ref_huff_select_query.argtypes = [vp, u64, u64]
        L.ref_huff_select_query.restype = u64
        self.L = L
        self.text = np.ascontiguousarray(text, dtype=np.uint8)
        self.h = L.ref_huff_new(_p(self.text), self.text.size)
        if not self.h:
            raise RuntimeError("reference wt_huff constructor failed")
        info = np.zeros(4, dtype=np.uint64)
        L.ref_huff_info(self.h, _p(info))
        self.n, self.sigma, self.size, nn = [int(x) for x in info]
        self.words = np.zeros((self.size + 63) // 64 + 1, dtype=np.uint64)
        L.ref_huff_bits(self.h, _p(self.words))
        self.words = self.words[: (self.size + 63) // 64]
        self.rank_tbl = np.zeros(max(L.ref_huff_rank_words(self.h), 1), dtype=np.uint64)
        L.ref_huff_rank(self.h, _p(self.rank_tbl))
        self.rank_tbl = self.rank_tbl[: L.ref_huff_rank_words(self.h)]
        self.nodes = np.zeros((max(nn, 1), 5), dtype=np.uint64)
        self.leaf = np.zeros(256, dtype=np.uint64)
        self.path = np.zeros(256, dtype=np.uint64)
        L.ref_huff_nodes(self.h, _p(self.nodes), _p(self.leaf), _p(self.path))
        self.nodes = self.nodes[:nn]

    def select_tables(self, t_b):
        info = np.zeros(8, dtype=np.uint64)
        self.L.ref_huff_select(self.h, t_b, _p(info), None, None, None)
        sb = np.zeros(max(int(info[6]), 1), dtype=np.uint64)
        desc = np.zeros(max(int(info[4]), 1), dtype=np.uint64)
        pool = np.zeros(max(int(info[7]), 1), dtype=np.uint64)
        self.L.ref_huff_select(self.h, t_b, _p(info), _p(sb), _p(desc), _p(pool))
        return info, sb[: int(info[6])], desc[: int(info[4])], pool[: int(info[7])]

    def access(self, i):
        return int(self.L.ref_huff_access(self.h, int(i)))

    def rank(self, i, c):
        return int(self.L.ref_huff_rank_query(self.h, int(i), int(c)))

    def select(self, i, c):
        return int(self.L.ref_huff_select_query(self.h, int(i), int(c)))

    def __del__(self):
        try:
            if self.h:
                self.L.ref_huff_free(self.h)
                self.h = None
        except Exception:
            pass


class RefWtInt:
    """The reference's own sdsl::wt_int (wt_int/wt_int_par.hpp), built by its
    constructor and queried through its member functions."""

    def __init__(self, sym, max_level, stream=None):
        L = _ref_wt_int()
        if stream is not None:  # wt_int::load of a serialized stream
            self.sym = None
            b = np.ascontiguousarray(stream, dtype=np.uint8)
            self.h = L.ref_wtint_load(_p(b), b.size)
            if not self.h:
                raise RuntimeError("reference wt_int::load failed")
        else:
            self.sym = np.ascontiguousarray(sym)
            self.h = L.ref_wtint_new(_p(self.sym), self.sym.dtype.itemsize, self.sym.size, max_level)
        if not self.h:
            raise RuntimeError("reference wt_int constructor failed")
        info = np.zeros(4, dtype=np.uint64)
        L.ref_wtint_info(self.h, _p(info))
        self.size, self.sigma, self.levels, nw = [int(x) for x in info]
        self.bits = np.zeros(max(nw, 1), dtype=np.uint64)
        L.ref_wtint_bits(self.h, _p(self.bits))
        self.bits = self.bits[:nw]

    @classmethod
    def load(cls, stream):
        """The reference's wt_int::load of a serialized stream."""
        return cls(None, 0, stream=stream)

    def serialize(self):
        """The reference's wt_int::serialize stream (uint8 array)."""
        L = _ref_wt_int()
        n = L.ref_wtint_serialize(self.h, None, 0)
        out = np.zeros(n, dtype=np.uint8)
        L.ref_wtint_serialize(self.h, _p(out), n)
        return out

    def access(self, i):
        return int(_ref_wt_int().ref_wtint_access(self.h, int(i)))

    def rank(self, i, c):
        return int(_ref_wt_int().ref_wtint_rank(self.h, int(i), int(c)))

    def select(self, i, c):
        return int(_ref_wt_int().ref_wtint_select(self.h, int(i), int(c)))

    def inverse_select(self, i):
        out = np.zeros(2, dtype=np.uint64)
        _ref_wt_int().ref_wtint_inverse_select(self.h, int(i), _p(out))
        return int(out[0]), int(out[1])

    def lex_count(self, i, j, c):
        out = np.zeros(3, dtype=np.uint64)
        _ref_wt_int().ref_wtint_lex_count(self.h, int(i), int(j), int(c), _p(out))
        return out

    def lex_smaller_count(self, i, c):
        out = np.zeros(2, dtype=np.uint64)
        _ref_wt_int().ref_wtint_lex_smaller_count(self.h, int(i), int(c), _p(out))
        return out

    def interval_symbols(self, i, j):
        cap = min(1 << self.levels, max(int(j) - int(i), 1))  # k <= j - i
        cs, ri, rj = (np.zeros(cap, dtype=np.uint64) for _ in range(3))
        k = _ref_wt_int().ref_wtint_interval_symbols(self.h, int(i), int(j), cap, _p(cs), _p(ri), _p(rj))
        return cs[:k], ri[:k], rj[:k]

    def range_search_2d(self, lb, rb, vlb, vrb, report=True):
        L = _ref_wt_int()
        cnt = L.ref_wtint_range_search_2d(self.h, int(lb), int(rb), int(vlb), int(vrb), 0, 0, None, None)
        if not report:
            return cnt, None, None
        pos = np.zeros(max(cnt, 1), dtype=np.uint64)
        val = np.zeros(max(cnt, 1), dtype=np.uint64)
        L.ref_wtint_range_search_2d(self.h, int(lb), int(rb), int(vlb), int(vrb), 1, cnt, _p(pos), _p(val))
        return cnt, pos[:cnt], val[:cnt]

    def expand(self, node):
        v = _u64(node)
        left, right = np.zeros(4, dtype=np.uint64), np.zeros(4, dtype=np.uint64)
        _ref_wt_int().ref_wtint_expand(self.h, _p(v), _p(left), _p(right))
        return left, right

    def expand_ranges(self, node, ranges):
        v, r = _u64(node), _u64(ranges).reshape(-1, 2)
        left, right = np.zeros_like(r), np.zeros_like(r)
        _ref_wt_int().ref_wtint_expand_ranges(self.h, _p(v), _p(r), r.shape[0], _p(left), _p(right))
        return left, right

    def __del__(self):
        try:
            if self.h:
                _ref_wt_int().ref_wtint_free(self.h)
                self.h = None
        except Exception:
            pass
