"""GPU wavelet-tree build parity: bits, node records, rank_support_v table and
select_support_mcl tables, bit-exact against the reference's golden vectors
and against the oracle on seeded inputs; wt_int queries against the oracle."""
import numpy as np
import pytest

import datagen
from helpers import GOLDEN, golden_ids, words_with_tail

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", GOLDEN, ids=golden_ids())
def test_matches_reference_golden(wtg, path):
    g = np.load(path)
    sym, sigma, L = g["sym"], int(g["sigma"]), int(g["levels"])
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    assert np.array_equal(t.bits(), g["bits"])
    ib = g["nodes"].dtype.itemsize
    nodes = t.nodes(2 * sigma, index_bytes=ib)
    assert np.array_equal(nodes[g["node_ids"]], g["nodes"])
    assert np.array_equal(t.rank_table(), g["rank"])
    for t_b in (0, 1):
        s = t.select_tables(t_b)
        info = [s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long, s.sb_nwords, s.pool_nwords]
        assert info == [int(x) for x in g[f"sel{t_b}_info"]]
        assert np.array_equal(s.sb_words, g[f"sel{t_b}_sb"])
        assert np.array_equal(s.desc, g[f"sel{t_b}_desc"])
        assert np.array_equal(s.pool, g[f"sel{t_b}_pool"])


def _gen(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "zipf8":
        return datagen.zipf_bytes(n, seed=seed), 8
    if kind == "acgt2":
        return rng.integers(0, 4, n).astype(np.uint8), 2
    if kind == "bin1":
        return rng.integers(0, 2, n).astype(np.uint8), 1
    if kind == "five3":
        return rng.integers(0, 5, n).astype(np.uint8), 3
    if kind == "u16_12":
        return rng.integers(0, 4096, n).astype(np.uint16), 12
    if kind == "exp20":
        return datagen.exp_u32(n, seed=seed), 20
    if kind == "u32_17":
        return rng.integers(0, 1 << 17, n).astype(np.uint32), 17
    if kind == "u64_20":
        return datagen.exp_u32(n, mean=2 ** 10, seed=seed).astype(np.uint64), 20
    if kind == "wide_u32_6":  # values above 2^levels: read through their low bits
        return rng.integers(0, 1 << 30, n).astype(np.uint32), 6
    if kind == "allsame":
        return np.full(n, 3, dtype=np.uint8), 2
    if kind == "sorted":
        return np.sort(rng.integers(0, 256, n)).astype(np.uint8), 8
    raise ValueError(kind)


CASES = [(k, n) for k in ("zipf8", "acgt2", "bin1", "five3", "exp20")
         for n in (1, 2, 31, 32, 33, 64, 65, 4095, 4096, 4097, 100003)]
CASES += [("u16_12", 77777), ("u32_17", 300001), ("u64_20", 50000), ("wide_u32_6", 70001),
          ("allsame", 123457), ("sorted", 262144), ("zipf8", 1 << 20), ("acgt2", (1 << 22) + 13),
          ("exp20", (1 << 20) + 7)]


def _expected(oracle, sym, L):
    n = sym.size
    bits, nodes = oracle.wt_build(sym, L, n_nodes=1 << L)
    w = words_with_tail(bits)
    return bits, nodes, w, oracle.rank_build(w, n * L)


@pytest.mark.parametrize("kind,n", CASES)
def test_build_matches_oracle(wtg, oracle, kind, n):
    sym, L = _gen(kind, n, seed=n + len(kind))
    bits, nodes, w, rank = _expected(oracle, sym, L)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    assert t.levels == L and t.n == n
    assert np.array_equal(t.bits(), bits)
    assert np.array_equal(t.nodes(1 << L, index_bytes=8), nodes)
    assert np.array_equal(t.rank_table(), rank)
    size = n * L
    for t_b in (0, 1):
        s = oracle.Select(w, size, t_b)
        g = t.select_tables(t_b)
        assert (g.arg_cnt, g.logn, g.logn4, g.nsb, g.has_long) == (s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long)
        assert np.array_equal(g.sb_words, s.sb_words)
        assert np.array_equal(g.desc, s.desc)
        assert np.array_equal(g.pool, s.pool)


@pytest.mark.parametrize("kind,n", [("zipf8", 100003), ("exp20", 200000), ("five3", 4097), ("u64_20", 30000),
                                    ("bin1", 65)])
def test_queries_match_oracle(wtg, oracle, kind, n):
    sym, L = _gen(kind, n, seed=7 * n)
    rng = np.random.default_rng(n)
    bits, _, w, rank = _expected(oracle, sym, L)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    idx = rng.integers(0, n, 4000).astype(np.uint64)
    assert np.array_equal(t.access(idx), sym[idx.astype(np.int64)].astype(np.uint64))
    assert np.array_equal(t.access(idx), oracle.wt_access(w, rank, n, L, idx))
    qi = rng.integers(0, n + 1, 4000).astype(np.uint64)
    qc = np.concatenate([sym[rng.integers(0, n, 3000)].astype(np.uint64),
                         rng.integers(0, 1 << L, 1000).astype(np.uint64)])
    assert np.array_equal(t.rank(qi, qc), oracle.wt_rank(w, rank, n, L, qi, qc))
    r, c = t.inverse_select(idx)
    assert np.array_equal(c, sym[idx.astype(np.int64)].astype(np.uint64))
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    cs = sym[rng.integers(0, n, 500)].astype(np.uint64)
    occ = {int(x): int(np.count_nonzero(sym == x)) for x in np.unique(cs)}
    ii = np.array([rng.integers(1, occ[int(x)] + 1) for x in cs], dtype=np.uint64)
    got = t.select(ii, cs)
    exp = np.array([oracle.wt_select(w, rank, s1, s0, n, L, int(i), int(x)) for i, x in zip(ii, cs)],
                   dtype=np.uint64)
    assert np.array_equal(got, exp)
    for k in range(0, 500, 50):
        j = int(got[k])
        assert sym[j] == cs[k] and r is not None
    # i beyond the occurrences of c -> UINT64_MAX (the reference throws)
    bad = t.select(np.array([n + 1], dtype=np.uint64), np.array([int(sym[0])], dtype=np.uint64))
    assert bad[0] == np.uint64(0xFFFFFFFFFFFFFFFF)


def test_empty_and_levels_derivation(wtg):
    t = wtg.WaveletTree(np.zeros(0, dtype=np.uint8), levels=3, flags=wtg.ALL)
    assert t.bit_words == 0 and np.array_equal(t.rank_table(), np.zeros(2, np.uint64))
    # levels = 0 derives wt_int's hi(max(1, max))+1 (wt_int_par.hpp:385-395)
    for mx, L in [(0, 1), (1, 1), (2, 2), (255, 8), (256, 9), ((1 << 20) - 1, 20)]:
        s = np.array([0, mx, mx // 2], dtype=np.uint32)
        assert wtg.WaveletTree(s, levels=0, flags=0).levels == L


def test_WT_shim_matches_reference_layout(wtg, oracle):
    sym = datagen.zipf_bytes(50000, seed=3)
    sym, sigma = oracle.remap_alphabet(sym)
    nodes, bits = wtg.WT(sym, sigma, index_bytes=4)
    L = oracle.levels_for_sigma(sigma)
    ob, on = oracle.wt_build(sym, L, n_nodes=2 * sigma)
    assert np.array_equal(bits, ob)
    on32 = on.astype(np.uint32)
    on32[on == np.uint64(0xFFFFFFFFFFFFFFFF)] = 0xFFFFFFFF
    assert np.array_equal(nodes, on32)


def test_remap_matches_oracle(wtg, oracle):
    for s in (np.frombuffer(b"ACGTNNACGT" * 100, dtype=np.uint8),
              datagen.exp_u32(100000, seed=9), np.array([5], dtype=np.uint16)):
        r1, s1 = wtg.remap_alphabet(s)
        r2, s2 = oracle.remap_alphabet(s)
        assert s1 == s2 and np.array_equal(r1, r2)


def test_rebuild_in_place_same_results(wtg):
    import torch
    sym = datagen.exp_u32(300000, seed=1)
    ref = wtg.WaveletTree(sym, levels=20, flags=wtg.ALL)
    d = torch.from_numpy(sym.view(np.int32)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    t = wtg.WaveletTree.from_device(d.data_ptr(), sym.size, 4, 20, wtg.ALL, stream)
    for _ in range(3):
        t = wtg.WaveletTree.from_device(d.data_ptr(), sym.size, 4, 20, wtg.ALL, stream, tree=t)
        t.sync()
        assert np.array_equal(t.bits(), ref.bits())
        assert np.array_equal(t.rank_table(), ref.rank_table())
        for t_b in (0, 1):
            a, b = t.select_tables(t_b), ref.select_tables(t_b)
            assert np.array_equal(a.pool, b.pool) and np.array_equal(a.desc, b.desc)


def test_large_properties(wtg):
    """Config-3 value distribution at 2^26 symbols: size-independent checks."""
    n, L = 1 << 26, 20
    sym = datagen.exp_u32(n, seed=123)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    rng = np.random.default_rng(5)
    idx = rng.integers(0, n, 1 << 16).astype(np.uint64)
    assert np.array_equal(t.access(idx), sym[idx.astype(np.int64)].astype(np.uint64))
    rank = t.rank_table()
    bits = t.bits()
    ones = int(np.unpackbits(bits.view(np.uint8)).sum())
    assert rank[-2] + ((rank[-1] >> np.uint64(54)) & np.uint64(0x1FF)) <= ones
    s1 = t.select_tables(1)
    assert s1.arg_cnt == ones
    hist = np.bincount(sym, minlength=1 << L)
    for c in (0, 1, 100, 16384, int(sym.max())):
        k = int(hist[c])
        if k:
            pos = t.select(np.array([1, k], dtype=np.uint64), np.array([c, c], dtype=np.uint64))
            assert sym[int(pos[0])] == c and sym[int(pos[1])] == c
            assert np.count_nonzero(sym[: int(pos[0])] == c) == 0
            assert t.rank(np.array([n], dtype=np.uint64), np.array([c], dtype=np.uint64))[0] == k


@pytest.mark.parametrize("kind,n", [("exp20", 100003), ("exp20", 1 << 20), ("five3", 4097), ("zipf8", 1 << 18),
                                    ("bin1", 65)])
def test_build_out_copies_equal_getters(wtg, kind, n):
    import torch
    sym, L = _gen(kind, n, seed=3 * n)
    ref = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    for pinned in (False, True):
        if pinned:
            bits_t = torch.zeros(ref.bit_words, dtype=torch.int64).pin_memory()
            rank_t = torch.zeros(ref.rank_words, dtype=torch.int64).pin_memory()
            bits, rank = bits_t.numpy().view(np.uint64), rank_t.numpy().view(np.uint64)
        else:
            bits = np.zeros(ref.bit_words, dtype=np.uint64)
            rank = np.zeros(ref.rank_words, dtype=np.uint64)
        t = wtg.WaveletTree.build_out(sym, L, wtg.ALL, bits.ctypes.data, rank.ctypes.data)
        assert np.array_equal(bits, ref.bits())
        assert np.array_equal(rank, ref.rank_table())
        # with n % 512 == 0 and a page-locked rank_dst the rank/select pass
        # runs level by level: every select table equals the one-pass build's
        for t_b in (0, 1):
            got, want = t.select_tables(t_b), ref.select_tables(t_b)
            assert (got.arg_cnt, got.nsb, got.has_long) == (want.arg_cnt, want.nsb, want.has_long)
            for f in ("sb_words", "desc", "pool"):
                assert np.array_equal(getattr(got, f), getattr(want, f)), (t_b, f)
        t.free()


@pytest.mark.parametrize("kind,n", [("exp20", 1 << 22), ("exp20", (1 << 22) + 777), ("zipf8", 3 * (1 << 21) + 5),
                                    ("u64_20", 1 << 22)])
def test_build_out_pinned_input_in_pieces(wtg, kind, n):
    """A page-locked input of at least 2^22 symbols is copied in pieces while
    the pre-pass counts each landed piece: every output equals the build from
    a pageable copy of the same input (one copy, then the pre-pass)."""
    import torch
    sym, L = _gen(kind, n, seed=n + 11)
    ref = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    as_int = {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[sym.dtype.itemsize]
    pinned = torch.from_numpy(sym.view(as_int)).pin_memory().numpy().view(sym.dtype)
    bits_t = torch.zeros(ref.bit_words, dtype=torch.int64).pin_memory()
    rank_t = torch.zeros(ref.rank_words, dtype=torch.int64).pin_memory()
    bits, rank = bits_t.numpy().view(np.uint64), rank_t.numpy().view(np.uint64)
    t = wtg.WaveletTree.build_out(pinned, L, wtg.ALL, bits.ctypes.data, rank.ctypes.data)
    assert np.array_equal(bits, ref.bits())
    assert np.array_equal(rank, ref.rank_table())
    assert np.array_equal(t.nodes(2 << L), ref.nodes(2 << L))
    for t_b in (0, 1):
        got, want = t.select_tables(t_b), ref.select_tables(t_b)
        for f in ("sb_words", "desc", "pool"):
            assert np.array_equal(getattr(got, f), getattr(want, f)), (t_b, f)
    # a rebuild of the same handle from the pinned input gives the same tree
    t = wtg.WaveletTree.build_out(pinned, L, wtg.ALL, bits.ctypes.data, rank.ctypes.data, tree=t)
    assert np.array_equal(bits, ref.bits())
    t.free()
