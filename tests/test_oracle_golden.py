"""The oracle reproduces the golden vectors made by the reference's own code
(WT() of levelWT, rank_support_v_par, select_support_mcl_par)."""
import numpy as np
import pytest

from helpers import GOLDEN, golden_ids, ref_nodes_u64, words_with_tail


@pytest.mark.parametrize("path", GOLDEN, ids=golden_ids())
def test_wt_bits_and_nodes(oracle, path):
    g = np.load(path)
    sym, sigma, L = g["sym"], int(g["sigma"]), int(g["levels"])
    for serial in (False, True):
        bits, nodes = oracle.wt_build(sym, L, n_nodes=2 * sigma, serial=serial)
        assert np.array_equal(bits, g["bits"])
        assert np.array_equal(nodes[g["node_ids"]], ref_nodes_u64(g))


@pytest.mark.parametrize("path", GOLDEN, ids=golden_ids())
def test_rank_and_select(oracle, path):
    g = np.load(path)
    size = g["sym"].size * int(g["levels"])
    words = words_with_tail(g["bits"])
    assert np.array_equal(oracle.rank_build(words, size), g["rank"])
    for t_b in (0, 1):
        for rule in (0, 1, 2):  # reference rule, forced init_slow, forced init_fast
            s = oracle.Select(words, size, t_b, rule)
            info = [s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long, s.sb_nwords, s.pool_nwords]
            assert info == [int(x) for x in g[f"sel{t_b}_info"]]
            assert np.array_equal(s.sb_words, g[f"sel{t_b}_sb"])
            assert np.array_equal(s.desc, g[f"sel{t_b}_desc"])
            assert np.array_equal(s.pool, g[f"sel{t_b}_pool"])
