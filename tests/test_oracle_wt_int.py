"""The oracle's wt_int queries reproduce the reference's own sdsl::wt_int
(wt_int/wt_int_par.hpp): the golden vectors of tests/golden/wt_int/ (made by
make_golden_wt_int.py from the reference), and, where the reference library
was compiled here, fresh seeded queries against it."""
import glob
import os

import numpy as np
import pytest

from helpers import NONE64, words_with_tail

WT_INT = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wt_int", "*.npz")))
IDS = [os.path.basename(p)[:-4] for p in WT_INT]


def tree_of(oracle, g):
    sym, L = g["sym"], int(g["levels"])
    n = sym.size
    bits, _ = oracle.wt_build(sym, L)
    w = words_with_tail(bits)
    rt = oracle.rank_build(w, n * L)
    return n, L, w, rt


def offsets(counts):
    return np.concatenate([[0], np.cumsum(counts.astype(np.int64))])


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_bits_and_point_queries(oracle, path):
    g = np.load(path)
    n, L, w, rt = tree_of(oracle, g)
    assert np.array_equal(w[: g["bits"].size], g["bits"])
    assert np.array_equal(oracle.wt_access(w, rt, n, L, g["access_i"]), g["access"])
    assert np.array_equal(oracle.wt_rank(w, rt, n, L, g["rank_i"], g["rank_c"]), g["rank"])
    inv = [oracle.wt_inverse_select(w, rt, n, L, i) for i in g["access_i"]]
    assert [r for r, _ in inv] == [int(x) for x in g["inv_rank"]]
    assert [c for _, c in inv] == [int(x) for x in g["inv_sym"]]
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    sel = [oracle.wt_select(w, rt, s1, s0, n, L, i, c) for i, c in zip(g["select_i"], g["select_c"])]
    assert np.array_equal(np.array(sel, dtype=np.uint64), g["select"])


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_lex_counts(oracle, path):
    g = np.load(path)
    n, L, w, rt = tree_of(oracle, g)
    assert np.array_equal(oracle.wt_lex_count(w, rt, n, L, g["lex_i"], g["lex_j"], g["lex_c"]), g["lex_count"])
    assert np.array_equal(oracle.wt_lex_smaller_count(w, rt, n, L, g["lex_i"], g["lex_c"]), g["lex_smaller"])


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_range_search_2d(oracle, path):
    g = np.load(path)
    n, L, w, rt = tree_of(oracle, g)
    lb, rb, vlb, vrb = g["r2d_lb"], g["r2d_rb"], g["r2d_vlb"], g["r2d_vrb"]
    assert np.array_equal(oracle.wt_range_count(w, rt, n, L, lb, rb, vlb, vrb), g["r2d_count"])
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    nr = int(g["r2d_report_q"])
    off = offsets(g["r2d_count"][:nr])
    for q in range(nr):
        p, v = oracle.wt_range_report(w, rt, s1, s0, n, L, lb[q], rb[q], vlb[q], vrb[q])
        assert np.array_equal(p, g["r2d_pos"][off[q]:off[q + 1]])
        assert np.array_equal(v, g["r2d_val"][off[q]:off[q + 1]])


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_interval_symbols(oracle, path):
    g = np.load(path)
    n, L, w, rt = tree_of(oracle, g)
    off = offsets(g["isym_k"])
    for q, (i, j) in enumerate(zip(g["isym_i"], g["isym_j"])):
        cs, ri, rj = oracle.wt_interval_symbols(w, rt, n, L, i, j)
        sl = slice(off[q], off[q + 1])
        assert np.array_equal(cs, g["isym_cs"][sl]) and np.array_equal(ri, g["isym_ri"][sl])
        assert np.array_equal(rj, g["isym_rj"][sl])


@pytest.mark.parametrize("path", WT_INT, ids=IDS)
def test_expand(oracle, path):
    g = np.load(path)
    n, L, w, rt = tree_of(oracle, g)
    for v, el, er in zip(g["exp_nodes"], g["exp_left"], g["exp_right"]):
        left, right = oracle.wt_expand(w, rt, n, v)
        assert np.array_equal(left, el) and np.array_equal(right, er)
    left, right = oracle.wt_expand_ranges(w, rt, g["expr_node"], g["expr_ranges"])
    assert np.array_equal(left, g["expr_left"]) and np.array_equal(right, g["expr_right"])


def test_select_past_count_is_none_in_golden():
    """The reference throws for select(i, c) past c's count; the fixtures
    record that as UINT64_MAX (and hold such cases)."""
    hits = sum(int((np.load(p)["select"] == NONE64).sum()) for p in WT_INT)
    assert hits > 0


def test_fresh_queries_against_reference(oracle):
    if not os.path.exists(os.path.join(os.path.dirname(oracle.__file__), "_ref", "libref_wt_int.so")):
        pytest.skip("the reference's wt_int was not compiled here")
    rng = np.random.default_rng(5)
    for n, L, top in ((3001, 7, 100), (999, 16, 1 << 16), (64, 2, 4)):
        sym = rng.integers(0, top, n).astype(np.uint32)
        R = oracle.RefWtInt(sym, L)
        w = words_with_tail(R.bits)
        rt = oracle.rank_build(w, n * L)
        s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
        for _ in range(150):
            i = int(rng.integers(0, n + 1))
            j = int(rng.integers(i, n + 1))
            c = int(rng.integers(0, (1 << L) + 2))
            assert np.array_equal(oracle.wt_lex_count(w, rt, n, L, [i], [j], [c])[0], R.lex_count(i, j, c))
            got = oracle.wt_interval_symbols(w, rt, n, L, i, j)
            assert all(np.array_equal(a, b) for a, b in zip(got, R.interval_symbols(i, j)))
            lb = int(rng.integers(0, n))
            rb = int(rng.integers(lb, n))
            vlb = int(rng.integers(0, 1 << L))
            vrb = int(rng.integers(vlb, (1 << L) + 3))
            cnt, p, v = R.range_search_2d(lb, rb, vlb, vrb)
            p2, v2 = oracle.wt_range_report(w, rt, s1, s0, n, L, lb, rb, vlb, vrb)
            assert cnt == p2.size and np.array_equal(p, p2) and np.array_equal(v, v2)
