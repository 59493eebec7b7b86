"""GPU rank_support_v / select_support_mcl over caller bitvectors: tables
bit-exact against the oracle (itself pinned to the reference's
rank_support_v_par / select_support_mcl_par), queries against the oracle."""
import numpy as np
import pytest

import datagen
from helpers import words_with_tail

pytestmark = pytest.mark.gpu

SIZES = [(0, 0.5), (1, 1.0), (1, 0.0), (63, 0.5), (64, 0.5), (65, 0.3), (511, 0.5), (512, 0.5), (513, 0.7),
         (1024, 0.1), (4096 * 3, 1.0), (99999, 0.05), (100000, 0.05), (100001, 0.5), (262144, 0.5),
         (524288, 0.003), (1000000, 0.001), (1000000, 0.999), (3000000, 0.0003), (1 << 21, 0.5),
         ((1 << 20) + 17, 0.0001), ((1 << 24) + 5, 0.01), (1 << 26, 0.3)]


@pytest.mark.parametrize("size,dens", SIZES)
def test_bitvector_tables(wtg, oracle, size, dens):
    words = datagen.random_bits(size, dens, seed=size ^ int(dens * 1000))
    w = words_with_tail(words)
    b = wtg.BitVectorSupport(words, size, wtg.ALL)
    assert np.array_equal(b.rank_table(), oracle.rank_build(w, size))
    rng = np.random.default_rng(size)
    for t_b in (0, 1):
        s = oracle.Select(w, size, t_b)
        g = b.select_tables(t_b)
        assert (g.arg_cnt, g.logn, g.logn4, g.nsb, g.has_long) == (s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long)
        assert np.array_equal(g.sb_words, s.sb_words)
        assert np.array_equal(g.desc, s.desc)
        assert np.array_equal(g.pool, s.pool)
        if s.arg_cnt:
            q = rng.integers(1, s.arg_cnt + 1, 20000).astype(np.uint64)
            assert np.array_equal(b.select(q, t_b), s.query_batch(q))
    idx = rng.integers(0, size + 1, 20000).astype(np.uint64)
    tbl = oracle.rank_build(w, size)
    exp = np.array([oracle.rank1(tbl, w, int(i)) for i in idx[:2000]], dtype=np.uint64)
    assert np.array_equal(b.rank(idx[:2000]), exp)


def test_garbage_past_size_is_ignored(wtg, oracle):
    size = 1000
    words = datagen.random_bits(size, 0.5, seed=1)
    dirty = words.copy()
    dirty[-1] |= np.uint64(0xFFFFFFFFFFFFFFFF) << np.uint64(size % 64)
    b = wtg.BitVectorSupport(dirty, size, wtg.ALL)
    w = words_with_tail(words)
    assert np.array_equal(b.rank_table(), oracle.rank_build(w, size))
    s = oracle.Select(w, size, 0)
    assert np.array_equal(b.select_tables(0).pool, s.pool)
