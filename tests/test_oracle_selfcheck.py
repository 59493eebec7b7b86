"""Oracle self-checks against naive definitions (rank = prefix popcount,
select = position of the i-th arg, wt access = the input symbol)."""
import numpy as np
import pytest

import datagen
from helpers import unpack_bits, words_with_tail

SIZES = [(0, 0.5), (1, 1.0), (63, 0.5), (64, 0.5), (511, 0.5), (512, 0.5), (513, 0.7), (4096 * 3, 1.0),
         (99999, 0.05), (100001, 0.5), (262144, 0.003), (300007, 0.999)]


@pytest.mark.parametrize("size,dens", SIZES)
def test_rank_select_naive(oracle, size, dens):
    w = words_with_tail(datagen.random_bits(size, dens, seed=size))
    bits = unpack_bits(w, size)
    tbl = oracle.rank_build(w, size)
    cum = np.concatenate([[0], np.cumsum(bits, dtype=np.int64)])
    idx = np.unique(np.concatenate([np.arange(0, size + 1, max(1, size // 997)), [size]]))
    assert all(oracle.rank1(tbl, w, int(i)) == cum[i] for i in idx)
    for t_b in (0, 1):
        s = oracle.Select(w, size, t_b)
        pos = np.flatnonzero(bits == t_b)
        assert s.arg_cnt == pos.size
        if pos.size:
            q = np.unique(np.linspace(1, pos.size, min(pos.size, 3000)).astype(np.uint64))
            assert np.array_equal(s.query_batch(q), pos[q.astype(np.int64) - 1].astype(np.uint64))


@pytest.mark.parametrize("n,sigma,dtype", [(1, 1, np.uint8), (1000, 3, np.uint8), (65536, 256, np.uint8),
                                           (20000, 1 << 12, np.uint32), (5000, 1 << 20, np.uint32)])
def test_wt_queries_naive(oracle, n, sigma, dtype):
    rng = np.random.default_rng(n)
    sym = rng.integers(0, sigma, n).astype(dtype)
    L = oracle.levels_for_sigma(sigma)
    bits, _ = oracle.wt_build(sym, L)
    w = words_with_tail(bits)
    tbl = oracle.rank_build(w, n * L)
    idx = rng.integers(0, n, 500).astype(np.uint64)
    assert np.array_equal(oracle.wt_access(w, tbl, n, L, idx), sym[idx.astype(np.int64)].astype(np.uint64))
    qi = rng.integers(0, n + 1, 300).astype(np.uint64)
    qc = sym[rng.integers(0, n, 300)].astype(np.uint64)
    exp = np.array([np.count_nonzero(sym[: int(i)] == c) for i, c in zip(qi, qc)], dtype=np.uint64)
    assert np.array_equal(oracle.wt_rank(w, tbl, n, L, qi, qc), exp)
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    for k in range(50):
        c = int(sym[rng.integers(0, n)])
        occ = np.flatnonzero(sym == c)
        i = int(rng.integers(1, occ.size + 1))
        assert oracle.wt_select(w, tbl, s1, s0, n, L, i, c) == occ[i - 1]
        j = int(rng.integers(0, n))
        r, cc = oracle.wt_inverse_select(w, tbl, n, L, j)
        assert cc == sym[j] and r == np.count_nonzero(sym[:j] == sym[j])


def test_remap_and_levels(oracle):
    s = np.frombuffer(b"ACGTNACGT", dtype=np.uint8)
    r, sigma = oracle.remap_alphabet(s)
    assert sigma == 5 and list(r) == [0, 1, 2, 4, 3, 0, 1, 2, 4]
    assert [oracle.levels_for_sigma(x) for x in (1, 2, 3, 4, 5, 256, 257, 1 << 20)] == [1, 1, 2, 2, 3, 8, 9, 20]
