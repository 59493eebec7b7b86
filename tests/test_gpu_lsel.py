"""Per-level select and the learned select index: every answer equals the
oracle's select_support_mcl (on the tree's concatenated bitvector, offset by
the args before the level) and the plain GPU route; each segment's recorded
window holds for every k (checked exhaustively in numpy); fallbacks, empty
levels, tiny trees and invalid queries."""
import numpy as np
import pytest

import datagen
from helpers import NONE64, unpack_bits, words_with_tail

pytestmark = pytest.mark.gpu


def _tree(wtg, oracle, sym, L):
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    bits, _ = oracle.wt_build(sym, L)
    return t, words_with_tail(bits)


def _level_bits(w, n, L):
    return unpack_bits(w, n * L).reshape(L, n) if n else np.zeros((L, 0), np.uint8)


def _queries(rng, lb, t_b, nq, extra_invalid=True):
    L, n = lb.shape
    m = (lb == t_b).sum(axis=1)
    lv = rng.integers(0, L, nq).astype(np.uint64)
    k = np.array([rng.integers(1, m[l] + 1) if m[l] else 1 for l in lv], dtype=np.uint64)
    if extra_invalid:
        lv = np.concatenate([lv, np.array([0, L - 1, L, L + 5], dtype=np.uint64)])
        k = np.concatenate([k, np.array([0, m[L - 1] + 1, 1, 1], dtype=np.uint64)])
    return lv, k


def _expected(oracle, w, lb, t_b, lv, k):
    L, n = lb.shape
    sel = oracle.Select(w, n * L, t_b)
    m = (lb == t_b).sum(axis=1)
    before = np.concatenate([[0], np.cumsum(m)])  # args before each level
    out = np.full(k.size, NONE64, dtype=np.uint64)
    ok = (lv < L)
    ok[ok] &= (k[ok] >= 1) & (k[ok] <= m[lv[ok].astype(np.int64)])
    li = lv[ok].astype(np.int64)
    g = sel.query_batch(before[li].astype(np.uint64) + k[ok])
    out[ok] = g - (li * n).astype(np.uint64)
    return out


def _check_windows(ls, lb, t_b):
    """For every level and every k: select(k) - pred(k) in [dlo, dhi]."""
    L, n = lb.shape
    for l in range(L):
        meta, rec = ls.level_model(t_b, l)
        pos = np.flatnonzero(lb[l] == t_b).astype(np.int64)
        assert meta["m"] == pos.size
        if pos.size == 0:
            assert meta["nseg"] == 0
            continue
        g = meta["g"]
        k0 = np.arange(pos.size, dtype=np.int64)  # k - 1
        seg = k0 >> g
        x = k0 - (seg << g)
        base, slope = rec[seg, 0].astype(np.int64), rec[seg, 1].astype(np.uint64)
        pred = base + ((slope * x.astype(np.uint64)) >> np.uint64(16)).astype(np.int64)
        err = pos - pred
        dlo, dhi = rec[seg, 2].view(np.int32).astype(np.int64), rec[seg, 3].view(np.int32).astype(np.int64)
        assert np.all(err >= dlo) and np.all(err <= dhi), (l, t_b)


CASES = [("exp20", 300001, 20, 1024), ("exp20", 1 << 18, 20, 1024), ("zipf8", 100003, 8, 1024),
         ("bin1", 65, 1, 1024), ("tiny5", 37, 5, 4), ("u16_12", 77777, 12, 64), ("allsame", 4099, 3, 1024),
         # n % 512 == 0: the levels start on superblocks and queries go through the compact rank directory
         ("zipf8", 1 << 17, 8, 1024), ("u16_12", 153600, 12, 64), ("bin1", 512, 1, 1024),
         ("exp20", 1 << 20, 20, 65536), ("tiny5", 1024, 5, 4), ("allsame", 4096, 3, 1024),
         # runs of 4096 equal bits: every 8192-bit directory block is half zeros, half ones, so
         # its superblock residuals overflow int8 and those queries take the plain select
         ("runs", 1 << 17, 1, 1024), ("runs", 300001, 2, 64)]


def _gen(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "exp20":
        return datagen.exp_u32(n, seed=seed)
    if kind == "zipf8":
        return datagen.zipf_bytes(n, seed=seed)
    if kind == "bin1":
        return rng.integers(0, 2, n).astype(np.uint8)
    if kind == "tiny5":
        return rng.integers(0, 32, n).astype(np.uint8)
    if kind == "u16_12":
        return rng.integers(0, 4096, n).astype(np.uint16)
    if kind == "allsame":
        return np.full(n, 5, dtype=np.uint8)
    if kind == "runs":
        return ((np.arange(n) // 4096) % 4).astype(np.uint8)
    raise ValueError(kind)


@pytest.mark.parametrize("kind,n,L,segments", CASES)
def test_learned_and_plain_level_select_match_oracle(wtg, oracle, kind, n, L, segments):
    sym = _gen(kind, n, seed=n + L)
    t, w = _tree(wtg, oracle, sym, L)
    lb = _level_bits(w, n, L)
    ls = wtg.LearnedSelect(t, segments=segments, samples=256)
    rng = np.random.default_rng(n)
    for t_b in (0, 1):
        lv, k = _queries(rng, lb, t_b, 20000)
        exp = _expected(oracle, w, lb, t_b, lv, k)
        assert np.array_equal(t.level_select(lv, k, t_b), exp)
        assert np.array_equal(ls.select(lv, k, t_b), exp)
        _check_windows(ls, lb, t_b)
    info = ls.info()
    assert info["misses"] == 0
    assert info["segments"] == sum(ls.level_model(tb, l)[0]["nseg"] for tb in (0, 1) for l in range(L))


@pytest.mark.parametrize("n", [5000, 5120])  # 5120 % 512 == 0: through the compact rank directory
def test_every_k_of_small_tree(wtg, oracle, n):
    sym = datagen.exp_u32(n, mean=2 ** 6, seed=11)
    L = 12
    t, w = _tree(wtg, oracle, sym, L)
    lb = _level_bits(w, sym.size, L)
    ls = wtg.LearnedSelect(t, segments=16, samples=8)
    for t_b in (0, 1):
        m = (lb == t_b).sum(axis=1)
        lv = np.concatenate([np.full(m[l], l) for l in range(L)]).astype(np.uint64)
        k = np.concatenate([np.arange(1, m[l] + 1) for l in range(L)]).astype(np.uint64)
        exp = _expected(oracle, w, lb, t_b, lv, k)
        assert np.array_equal(ls.select(lv, k, t_b), exp)
        assert np.array_equal(t.level_select(lv, k, t_b), exp)


@pytest.mark.parametrize("n", [200000, 204800])
def test_fallback_paths_stay_exact(wtg, oracle, n):
    sym = datagen.exp_u32(n, seed=5)
    L = 20
    t, w = _tree(wtg, oracle, sym, L)
    lb = _level_bits(w, sym.size, L)
    # two segments per level and a 64-position window: most segments fall back
    ls = wtg.LearnedSelect(t, segments=2, samples=64, max_window=64)
    info = ls.info()
    assert info["fallback_segments"] > 0
    rng = np.random.default_rng(3)
    for t_b in (0, 1):
        lv, k = _queries(rng, lb, t_b, 20000)
        assert np.array_equal(ls.select(lv, k, t_b), _expected(oracle, w, lb, t_b, lv, k))
    assert ls.info()["misses"] == 0


def test_stale_index_after_rebuild_is_rejected(wtg):
    import torch
    sym = datagen.exp_u32(100000, seed=1)
    d = torch.from_numpy(sym.view(np.int32)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    t = wtg.WaveletTree.from_device(d.data_ptr(), sym.size, 4, 20, wtg.ALL, stream)
    t.sync()
    ls = wtg.LearnedSelect(t)
    assert ls.select(np.array([10]), np.array([1]), 0)[0] != NONE64
    wtg.WaveletTree.from_device(d.data_ptr(), sym.size, 4, 20, wtg.ALL, stream, tree=t)
    t.sync()
    with pytest.raises(wtg.WtgError):
        ls.select(np.array([10]), np.array([1]), 0)


def test_device_query_entry_points(wtg, oracle):
    import torch
    sym = datagen.exp_u32(1 << 16, seed=9)
    L = 20
    t, w = _tree(wtg, oracle, sym, L)
    lb = _level_bits(w, sym.size, L)
    ls = wtg.LearnedSelect(t)
    rng = np.random.default_rng(4)
    lv, k = _queries(rng, lb, 1, 5000, extra_invalid=False)
    exp = _expected(oracle, w, lb, 1, lv, k)
    dl = torch.from_numpy(lv.view(np.int64)).cuda()
    dk = torch.from_numpy(k.view(np.int64)).cuda()
    o1 = torch.empty_like(dk)
    o2 = torch.empty_like(dk)
    s = torch.cuda.current_stream().cuda_stream
    ls.select_device(1, dl.data_ptr(), dk.data_ptr(), k.size, o1.data_ptr(), s)
    t.level_select_device(1, dl.data_ptr(), dk.data_ptr(), k.size, o2.data_ptr(), s)
    torch.cuda.synchronize()
    assert np.array_equal(o1.cpu().numpy().view(np.uint64), exp)
    assert np.array_equal(o2.cpu().numpy().view(np.uint64), exp)


def test_index_outliving_its_tree_fails_cleanly(wtg):
    sym = datagen.exp_u32(50000, seed=2)
    t = wtg.WaveletTree(sym, levels=20, flags=wtg.ALL)
    ls = wtg.LearnedSelect(t)
    t.free()
    with pytest.raises(wtg.WtgError):
        ls.select(np.array([3]), np.array([1]), 1)
    assert ls.info()["segments"] > 0
    ls.free()
