"""Huffman-shaped wavelet tree, CPU side: the oracle's restatement of the
reference's wt_huff build (wt_huff/wt_huff_par.hpp:82-117,
wt_huff/wt_pc_par.hpp:193-258,321-361) and its queries (:430-552) equal the
reference's own outputs (golden fixtures made by the reference, and the live
reference where it builds here)."""
import glob
import os

import numpy as np
import pytest

import datagen

HUFF = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "huff", "*.npz")))


def _ids():
    return [os.path.basename(p)[:-4] for p in HUFF]


def _ref_nodes(g):
    nd = g["nodes"].astype(np.int64)
    nd[nd == 0xFFFF] = -1
    return nd


def check_against(o, g):
    """o: an object with words/rank table/shape/select tables; g: golden arrays."""
    sh = o.shape
    assert sh.bv_size == int(g["size"]) and sh.sigma == int(g["sigma"])
    assert np.array_equal(o.words[: g["words"].size], g["words"])
    assert np.array_equal(o.rank_tbl, g["rank"])
    nd = _ref_nodes(g)
    assert np.array_equal(sh.nodes[:, 0], nd[:, 0])       # bv_pos
    assert np.array_equal(sh.nodes[:, 3:6], nd[:, 2:5])   # parent, children
    assert np.array_equal(o.node_rank, g["nodes"][:, 1])  # bv_pos_rank (symbol of a leaf)
    assert np.array_equal(sh.path, g["path"] & np.uint64((1 << 56) - 1))
    assert np.array_equal(sh.plen, (g["path"] >> np.uint64(56)).astype(np.int64))
    for t_b in (0, 1):
        s = o.sel[t_b]
        assert [s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long, s.sb_nwords, s.pool_nwords] == \
               [int(x) for x in g[f"sel{t_b}_info"]]
        assert np.array_equal(s.sb_words, g[f"sel{t_b}_sb"])
        assert np.array_equal(s.desc, g[f"sel{t_b}_desc"])
        assert np.array_equal(s.pool, g[f"sel{t_b}_pool"])


@pytest.mark.parametrize("path", HUFF, ids=_ids())
def test_oracle_matches_reference_golden(oracle, path):
    g = np.load(path)
    o = oracle.HuffOracle(g["text"])
    check_against(o, g)
    assert [o.access(int(i)) for i in g["acc_i"]] == [int(x) for x in g["acc"]]
    assert [o.rank(int(i), int(c)) for i, c in zip(g["rank_i"], g["rank_c"])] == [int(x) for x in g["rank_ans"]]
    assert [o.select(int(i), int(c)) for i, c in zip(g["sel_i"], g["sel_c"])] == [int(x) for x in g["sel_ans"]]


@pytest.mark.parametrize("kind,n", [("zipf", 200003), ("dna", 50000), ("bytes", 7), ("two", 129)])
def test_oracle_matches_live_reference(oracle, kind, n):
    if not oracle.ref_available("wt_huff"):
        pytest.skip("the reference checkout is not built here")
    rng = np.random.default_rng(n)
    text = {"zipf": lambda: datagen.zipf_bytes(n, seed=n), "dna": lambda: datagen.dna_markov(n, seed=n),
            "bytes": lambda: rng.integers(0, 256, n).astype(np.uint8),
            "two": lambda: rng.integers(0, 2, n).astype(np.uint8)}[kind]()
    R, o = oracle.RefWtHuff(text), oracle.HuffOracle(text)
    assert np.array_equal(o.words[: R.words.size], R.words)
    assert np.array_equal(o.rank_tbl, R.rank_tbl)
    for i in range(0, n, max(1, n // 50)):
        assert o.access(i) == R.access(i) == int(text[i])
