"""sdsl serialize() streams from the GPU structures, through the C ABI:
byte for byte equal to the streams the reference's own wt_int,
rank_support_v and select_support_mcl wrote (golden fixtures), and to the
oracle's restatement on larger seeded inputs (long superblocks, init_slow
and init_fast sizes, a 2^24-symbol byte text), as the reference's own check
compares serialized structures (wt_int/compareResults.py:1-15)."""
import numpy as np
import pytest

import datagen
from test_oracle_serialize import BV, WT, _ids

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", WT, ids=_ids(WT))
def test_tree_stream_matches_reference_golden(wtg, path):
    g = np.load(path)
    sym, L = g["sym"], int(g["levels"])
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    assert np.array_equal(t.serialize(), g["stream"])
    t.free()


@pytest.mark.parametrize("path", BV, ids=_ids(BV))
def test_support_streams_match_reference_golden(wtg, path):
    g = np.load(path)
    b = wtg.BitVectorSupport(g["words"], int(g["size"]), wtg.ALL)
    assert np.array_equal(b.serialize(wtg.RANK), g["rank"])
    assert np.array_equal(b.serialize(wtg.SELECT1), g["sel1"])
    assert np.array_equal(b.serialize(wtg.SELECT0), g["sel0"])
    b.free()


@pytest.mark.parametrize("kind,n,L", [("zipf", 1 << 24, 8), ("exp", (1 << 22) + 9, 20), ("exp", 5000, 20),
                                      ("exp", 4999, 20), ("sparse", 1 << 21, 18), ("one", 3000, 2)])
def test_tree_stream_matches_oracle(wtg, oracle, kind, n, L):
    rng = np.random.default_rng(n + L)
    if kind == "zipf":
        sym = datagen.zipf_bytes(n, seed=n)
    elif kind == "exp":
        sym = datagen.exp_u32(n, seed=n)
    elif kind == "sparse":  # mostly zeros: select1 takes long superblocks
        sym = np.zeros(n, dtype=np.uint32)
        sym[rng.choice(n, 2000, replace=False)] = rng.integers(1, 1 << L, 2000)
    else:
        sym = np.full(n, 2, dtype=np.uint8)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    got = t.serialize()
    exp = oracle.serialize_wt_int(sym, L)
    assert got.size == exp.size
    assert np.array_equal(got, exp)
    mask = (1 << L) - 1
    assert t.sigma() == np.unique(sym.astype(np.uint64) & np.uint64(mask)).size
    if kind == "sparse":
        assert t.select_tables(1).has_long == 1
    t.free()


@pytest.mark.parametrize("size,dens", [((1 << 23) + 5, 0.0002), (1 << 22, 0.5), (100001, 0.99), (777, 0.1)])
def test_support_streams_match_oracle(wtg, oracle, size, dens):
    words = datagen.random_bits(size, dens, seed=size)
    w = np.concatenate([words, np.zeros(1, np.uint64)])
    b = wtg.BitVectorSupport(words, size, wtg.ALL)
    assert np.array_equal(b.serialize(wtg.RANK), oracle.serialize_rank(oracle.rank_build(w, size)))
    for t_b, part in ((1, wtg.SELECT1), (0, wtg.SELECT0)):
        assert np.array_equal(b.serialize(part), oracle.serialize_select(oracle.Select(w, size, t_b)))
    b.free()


def test_stream_needs_all_supports(wtg):
    t = wtg.WaveletTree(np.arange(100, dtype=np.uint8), levels=7, flags=wtg.RANK)
    with pytest.raises(wtg.WtgError) as e:
        t.serialize()
    assert e.value.code == wtg.ERR_INVALID
    t.free()
