"""sdsl serialize() streams, CPU side: the oracle's restatement of the byte
format equals the streams the reference's own wt_int, rank_support_v and
select_support_mcl wrote (golden fixtures), and -- where the reference
builds here -- equals the live reference on fresh inputs, and the
reference's own load() reads the oracle's streams back."""
import glob
import os

import numpy as np
import pytest

import datagen

SER = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "serialize", "*.npz")))
WT = [p for p in SER if os.path.basename(p).startswith("wt_")]
BV = [p for p in SER if os.path.basename(p).startswith("bv_")]


def _ids(paths):
    return [os.path.basename(p)[:-4] for p in paths]


@pytest.mark.parametrize("path", WT, ids=_ids(WT))
def test_wt_int_stream_matches_reference_golden(oracle, path):
    g = np.load(path)
    sym, L = g["sym"], int(g["levels"])
    if L == 0:  # wt_int derives max_level = hi(max(1, max symbol)) + 1
        L = oracle.hi(max(1, int(sym.max()) if sym.size else 1)) + 1
    assert np.array_equal(oracle.serialize_wt_int(sym, L), g["stream"])


@pytest.mark.parametrize("path", BV, ids=_ids(BV))
def test_support_streams_match_reference_golden(oracle, path):
    g = np.load(path)
    size = int(g["size"])
    w = np.concatenate([g["words"], np.zeros(1, np.uint64)])
    assert np.array_equal(oracle.serialize_rank(oracle.rank_build(w, size)), g["rank"])
    for t_b in (0, 1):
        assert np.array_equal(oracle.serialize_select(oracle.Select(w, size, t_b)), g[f"sel{t_b}"])


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available("wt_int") or not oracle.ref_available("rank_select"):
        pytest.skip("the reference checkout is not built here")
    return oracle


@pytest.mark.parametrize("n,L,seed", [(1, 1, 1), (65, 3, 2), (4097, 20, 3), (123457, 17, 4)])
def test_live_reference_streams_and_load(ref, n, L, seed):
    sym = datagen.exp_u32(n, mean=2 ** (L - 3) if L > 3 else 1, seed=seed)
    R = ref.RefWtInt(sym, L)
    stream = ref.serialize_wt_int(sym, L)
    assert np.array_equal(R.serialize(), stream)
    back = ref.RefWtInt.load(stream)  # the reference's wt_int::load of the oracle's stream
    mask = (1 << L) - 1
    for i in range(0, n, max(1, n // 97)):
        assert back.access(i) == int(sym[i]) & mask
    c = int(sym[0]) & mask
    assert back.rank(n, c) == int(np.count_nonzero((sym.astype(np.int64) & mask) == c))
