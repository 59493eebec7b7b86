"""wt_int's range queries on the GPU (lex_count, lex_smaller_count,
range_search_2d, interval_symbols, expand), through the C ABI: bit-exact
against the reference's own wt_int answers (tests/golden/wt_int/), against the
oracle on seeded inputs with invalid bounds mixed in, and size-independent
properties at 2^24 symbols."""
import glob
import os

import numpy as np
import pytest

import datagen
from helpers import NONE64, words_with_tail

pytestmark = pytest.mark.gpu

WT_INT = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wt_int", "*.npz")))
IDS = [os.path.basename(p)[:-4] for p in WT_INT]


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_matches_reference_wt_int(wtg, path):
    g = np.load(path)
    sym, L = g["sym"], int(g["levels"])
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    assert np.array_equal(t.bits(), g["bits"])
    # point queries
    assert np.array_equal(t.access(g["access_i"]), g["access"])
    assert np.array_equal(t.rank(g["rank_i"], g["rank_c"]), g["rank"])
    r, c = t.inverse_select(g["access_i"])
    assert np.array_equal(r, g["inv_rank"]) and np.array_equal(c, g["inv_sym"])
    assert np.array_equal(t.select(g["select_i"], g["select_c"]), g["select"])
    # lex counts
    assert np.array_equal(t.lex_count(g["lex_i"], g["lex_j"], g["lex_c"]), g["lex_count"])
    assert np.array_equal(t.lex_smaller_count(g["lex_i"], g["lex_c"]), g["lex_smaller"])
    # range_search_2d: counts of all queries, points of the first half
    lb, rb, vlb, vrb = g["r2d_lb"], g["r2d_rb"], g["r2d_vlb"], g["r2d_vrb"]
    assert np.array_equal(t.range_count(lb, rb, vlb, vrb), g["r2d_count"])
    nr = int(g["r2d_report_q"])
    cnt, off, pos, val = t.range_search_2d(lb[:nr], rb[:nr], vlb[:nr], vrb[:nr])
    assert np.array_equal(cnt, g["r2d_count"][:nr])
    assert np.array_equal(pos, g["r2d_pos"]) and np.array_equal(val, g["r2d_val"])
    # interval_symbols
    k, off, cs, ri, rj = t.interval_symbols(g["isym_i"], g["isym_j"])
    assert np.array_equal(k, g["isym_k"])
    assert np.array_equal(cs, g["isym_cs"]) and np.array_equal(ri, g["isym_ri"])
    assert np.array_equal(rj, g["isym_rj"])
    # expand
    left, right = t.expand(g["exp_nodes"])
    assert np.array_equal(left, g["exp_left"]) and np.array_equal(right, g["exp_right"])
    left, right = t.expand_ranges(g["expr_node"], g["expr_ranges"])
    assert np.array_equal(left, g["expr_left"]) and np.array_equal(right, g["expr_right"])


def _tree(wtg, oracle, sym, L):
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    bits, _ = oracle.wt_build(sym, L)
    w = words_with_tail(bits)
    return t, w, oracle.rank_build(w, sym.size * L)


CASES = [("exp_u32", 1 << 18, 20), ("zipf_u8", 300007, 8), ("rand_u16", 100003, 16), ("bin_u8", 4099, 1),
         ("rand_u32", 70001, 24)]


def _gen(kind, n):
    rng = np.random.default_rng(n)
    if kind == "exp_u32":
        return datagen.exp_u32(n, seed=n)
    if kind == "zipf_u8":
        return datagen.zipf_bytes(n, seed=3)
    if kind == "rand_u16":
        return rng.integers(0, 1 << 16, n).astype(np.uint16)
    if kind == "bin_u8":
        return rng.integers(0, 2, n).astype(np.uint8)
    return rng.integers(0, 1 << 24, n).astype(np.uint32)


@pytest.mark.parametrize("kind,n,L", CASES)
def test_counts_match_oracle(wtg, oracle, kind, n, L):
    sym = _gen(kind, n)
    t, w, rt = _tree(wtg, oracle, sym, L)
    rng = np.random.default_rng(n + 1)
    nq = 20000
    top = 1 << L
    i = rng.integers(0, n + 1, nq).astype(np.uint64)
    j = np.minimum(n, i + rng.integers(0, n + 1, nq) // rng.integers(1, 1000, nq)).astype(np.uint64)
    c = np.where(rng.integers(0, 3, nq) == 0, rng.integers(0, top + 4, nq), sym[rng.integers(0, n, nq)])
    c = c.astype(np.uint64)
    # invalid bounds: i > j, j > n
    i[:5], j[:5] = j[:5] + 1, j[:5]
    j[5:10] = n + 1
    got = t.lex_count(i, j, c)
    ok = (i <= j) & (j <= n)
    assert np.array_equal(got[ok], oracle.wt_lex_count(w, rt, n, L, i[ok], j[ok], c[ok]))
    assert np.all(got[~ok] == NONE64)
    ok2 = i <= n
    got2 = t.lex_smaller_count(i, c)
    assert np.array_equal(got2[ok2], oracle.wt_lex_smaller_count(w, rt, n, L, i[ok2], c[ok2]))
    # range counts
    lb = rng.integers(0, n, nq).astype(np.uint64)
    rb = np.minimum(n - 1, lb + rng.integers(0, n, nq) // rng.integers(1, 100, nq)).astype(np.uint64)
    vlb = rng.integers(0, top + 2, nq).astype(np.uint64)
    vrb = (vlb + rng.integers(0, top + 8, nq) // rng.integers(1, 64, nq)).astype(np.uint64)
    vlb[:50] = top  # the reference's boundary: vlb = vrb = 2^L after clamping
    rb[50:60] = n  # invalid
    got = t.range_count(lb, rb, vlb, vrb)
    ok = ~((lb <= rb) & (rb >= n))
    exp = oracle.wt_range_count(w, rt, n, L, lb[ok], rb[ok], vlb[ok], vrb[ok])
    assert np.array_equal(got[ok], exp)
    assert np.all(got[~ok] == NONE64)


@pytest.mark.parametrize("kind,n,L", CASES)
def test_report_and_symbols_match_oracle(wtg, oracle, kind, n, L):
    sym = _gen(kind, n)
    t, w, rt = _tree(wtg, oracle, sym, L)
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    rng = np.random.default_rng(n + 2)
    nq = 300
    top = 1 << L
    lb = rng.integers(0, n, nq).astype(np.uint64)
    rb = np.minimum(n - 1, lb + rng.integers(0, 4000, nq)).astype(np.uint64)
    vlb = rng.integers(0, top, nq).astype(np.uint64)
    vrb = (vlb + rng.integers(0, top + 8, nq) // rng.integers(1, 8, nq)).astype(np.uint64)
    rb[:3] = n  # invalid: no points
    cnt, off, pos, val = t.range_search_2d(lb, rb, vlb, vrb)
    for q in range(nq):
        if q < 3:
            assert cnt[q] == NONE64 and off[q + 1] == off[q]
            continue
        p, v = oracle.wt_range_report(w, rt, s1, s0, n, L, lb[q], rb[q], vlb[q], vrb[q])
        assert np.array_equal(pos[off[q]:off[q + 1]], p) and np.array_equal(val[off[q]:off[q + 1]], v), q
    # a cap keeps the first points in the same order
    cap = int(off[-1]) // 2
    _, _, pos2, val2 = t.range_search_2d(lb, rb, vlb, vrb, cap=cap)
    assert np.array_equal(pos2, pos[:cap]) and np.array_equal(val2, val[:cap])
    # interval_symbols
    i = rng.integers(0, n + 1, nq).astype(np.uint64)
    j = np.minimum(n, i + rng.integers(0, 3000, nq)).astype(np.uint64)
    j[:3] = n + 1
    k, off, cs, ri, rj = t.interval_symbols(i, j)
    for q in range(nq):
        if q < 3:
            assert k[q] == NONE64
            continue
        a, b, c = oracle.wt_interval_symbols(w, rt, n, L, i[q], j[q])
        sl = slice(off[q], off[q + 1])
        assert np.array_equal(cs[sl], a) and np.array_equal(ri[sl], b) and np.array_equal(rj[sl], c), q


def test_empty_and_degenerate_queries(wtg):
    sym = np.array([3, 1, 3, 0, 2, 3, 1], dtype=np.uint8)
    t = wtg.WaveletTree(sym, levels=2, flags=wtg.ALL)
    assert t.lex_count([], [], []).shape == (0, 3)
    k, off, cs, _, _ = t.interval_symbols([2, 0], [2, 7])
    assert list(k) == [0, 4] and list(cs) == [0, 1, 2, 3]
    cnt, _, pos, val = t.range_search_2d([4], [3], [0], [3])  # lb > rb
    assert list(cnt) == [0] and pos.size == 0
    cnt, _, pos, val = t.range_search_2d([0], [6], [3], [1])  # vlb > vrb
    assert list(cnt) == [0]
    cnt, _, pos, val = t.range_search_2d([0], [6], [3], [3])
    assert list(pos) == [0, 2, 5] and list(val) == [3, 3, 3]
    left, right = t.expand(np.array([[0, 7, 2, 0]], dtype=np.uint64))  # a leaf
    assert np.all(left == NONE64) and np.all(right == NONE64)


def test_properties_at_scale(wtg):
    """2^24 symbols, 20 levels: counts partition their ranges."""
    n, L = 1 << 24, 20
    sym = datagen.exp_u32(n, seed=17)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    rng = np.random.default_rng(8)
    nq = 1 << 16
    i = rng.integers(0, n + 1, nq).astype(np.uint64)
    j = np.minimum(n, i + rng.integers(0, n, nq) // rng.integers(1, 1 << 12, nq)).astype(np.uint64)
    c = sym[rng.integers(0, n, nq)].astype(np.uint64)
    lc = t.lex_count(i, j, c)
    occ = t.rank(j, c) - t.rank(i, c)
    assert np.array_equal(lc[:, 0], t.rank(i, c))
    assert np.array_equal(lc[:, 1] + lc[:, 2] + occ, j - i)
    ls = t.lex_smaller_count(j, c)
    assert np.array_equal(ls[:, 1] - t.lex_smaller_count(i, c)[:, 1], lc[:, 1])
    # full value range counts every position; a split at c adds up
    rb = np.maximum(j, np.uint64(1)) - np.uint64(1)
    lb = np.minimum(i, rb)
    full = t.range_count(lb, rb, np.zeros(nq, np.uint64), np.full(nq, 1 << L, np.uint64))
    assert np.array_equal(full, rb - lb + 1)
    lo = t.range_count(lb, rb, np.zeros(nq, np.uint64), np.maximum(c, 1) - 1)
    hi = t.range_count(lb, rb, np.maximum(c, 1), np.full(nq, (1 << L) - 1, np.uint64))
    assert np.array_equal(lo + hi, full)
    # interval_symbols: distinct increasing symbols whose occurrences add up
    sel = slice(0, 2000)
    k, off, cs, ri, rj = t.interval_symbols(i[sel], j[sel])
    per = np.array([int((rj[off[q]:off[q + 1]] - ri[off[q]:off[q + 1]]).sum()) for q in range(k.size)])
    assert np.array_equal(per, (j[sel] - i[sel]).astype(np.int64))
    assert all(np.all(np.diff(cs[off[q]:off[q + 1]].astype(np.int64)) > 0) for q in range(k.size))


def test_device_entry_points(wtg, oracle):
    import torch
    sym = datagen.exp_u32(1 << 16, seed=4)
    n, L = sym.size, 20
    t, w, rt = _tree(wtg, oracle, sym, L)
    rng = np.random.default_rng(1)
    nq = 4096
    i = rng.integers(0, n + 1, nq).astype(np.uint64)
    j = np.minimum(n, i + rng.integers(0, 5000, nq)).astype(np.uint64)
    c = sym[rng.integers(0, n, nq)].astype(np.uint64)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()

    di, dj, dc = dev(i), dev(j), dev(c)
    o = [torch.empty_like(di) for _ in range(3)]
    s = torch.cuda.current_stream().cuda_stream
    t.lex_count_device(di.data_ptr(), dj.data_ptr(), dc.data_ptr(), nq, o[0].data_ptr(), o[1].data_ptr(),
                       o[2].data_ptr(), s)
    dcnt = torch.empty_like(di)
    top = np.full(nq, (1 << L) - 1, np.uint64)
    rbm = np.maximum(j, 1) - 1
    dtop, drb = dev(top), dev(rbm)
    t.range_count_device(di.data_ptr(), drb.data_ptr(), dc.data_ptr(), dtop.data_ptr(), nq, dcnt.data_ptr(), s)
    torch.cuda.synchronize()
    got = np.stack([x.cpu().numpy().view(np.uint64) for x in o], axis=1)
    assert np.array_equal(got, oracle.wt_lex_count(w, rt, n, L, i, j, c))
    exp = oracle.wt_range_count(w, rt, n, L, i, rbm, c, top)
    assert np.array_equal(dcnt.cpu().numpy().view(np.uint64), exp)
