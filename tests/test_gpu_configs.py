"""Bit-exact parity at the measured workloads' own sizes, against the oracle.

The other GPU parity tests stop at a few million symbols; some decisions of
the reference's rank/select construction only occur at full size (the
select_support_mcl widths and the long/mini rule at log n = 35, log^4 n =
1 500 625 for the 20 * 2^30-bit level bitvector, select/select_support_mcl_par.hpp:
619-636; the rank table's final pair when the capacity is a multiple of 512,
rank/rank_support_v_par.hpp:95-113).  Every word of the level bits, the
reachable node records, the rank table and both select structures is
compared here:

  * byte text: n = 2^24 Zipf(1.0) bytes, 8 levels;
  * integer tree: n = 2^30 uint32, Exp(mean 2^14) clamped to 2^20 - 1,
    20 levels (about 25 GB of host memory and a minute of host time);
  * FM-index: the 3-level tree of the BWT of a 2^28-symbol order-2 Markov DNA
    text (suffix order checked in full, counts against the oracle's backward
    search);
  * batch: every text of a 4096-text plan (lengths floor(2^U[10, 20]), 2
    levels) against the oracle's per-text build.
"""
import numpy as np
import pytest

import datagen

pytestmark = pytest.mark.gpu


def _compare_tree(oracle, t, sym, L, n_nodes):
    """GPU tree t against the oracle's build of sym with L levels."""
    n = sym.size
    w, nodes = oracle.wt_build(sym, L, n_nodes=n_nodes, tail=True)
    got = t.bits()
    assert got.size == w.size - 1
    assert np.array_equal(got, w[:-1]), "level bits"
    del got
    assert np.array_equal(t.nodes(n_nodes, index_bytes=8), nodes), "node records"
    del nodes
    rank = oracle.rank_build(w, n * L)
    got = t.rank_table()
    assert np.array_equal(got, rank), "rank table"
    del got, rank
    infos = []
    for t_b in (0, 1):
        s = oracle.Select(w, n * L, t_b)
        g = t.select_tables(t_b)
        info = (g.size, g.arg_cnt, g.logn, g.logn4, g.nsb, g.has_long, g.sb_nwords, g.pool_nwords)
        assert info == (s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long, s.sb_nwords, s.pool_nwords), t_b
        assert np.array_equal(g.sb_words, s.sb_words), ("select superblocks", t_b)
        assert np.array_equal(g.desc, s.desc), ("select descriptors", t_b)
        assert np.array_equal(g.pool, s.pool), ("select blocks", t_b)
        infos.append(info)
        del s, g
    return infos


def test_byte_text_2p24_zipf_8_levels(wtg, oracle):
    sym = datagen.zipf_bytes(1 << 24, seed=101)
    t = wtg.WaveletTree(sym, levels=8, flags=wtg.ALL)
    infos = _compare_tree(oracle, t, sym, 8, 1 << 8)
    assert infos[1][2] == 28  # logn = hi(2^27) + 1
    t.free()


def test_integer_tree_2p30_exp_20_levels(wtg, oracle):
    n, L = 1 << 30, 20
    sym = datagen.exp_u32(n, seed=103)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    t.sync()
    infos = _compare_tree(oracle, t, sym, L, 1 << L)
    for size, _, logn, logn4, _, _, _, _ in infos:
        assert size == n * L and logn == 35 and logn4 == 35 ** 4
    # the top levels are nearly all zeros: select1 takes long superblocks
    assert infos[1][5] == 1
    # final rank pair when the capacity is a multiple of 512: (total, 0)
    rank_tail = t.rank_table()[-2:]
    assert rank_tail[1] == 0 and rank_tail[0] == infos[1][1]
    t.free()


def test_fm_index_bwt_2p28(wtg, oracle):
    torch = pytest.importorskip("torch")
    n, dev = 1 << 28, torch.device("cuda")
    text = datagen.dna_markov_device(n, torch, dev, seed=107)
    sa = torch.empty(n, dtype=torch.int32, device=dev)
    bw = torch.empty(n, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    wtg.suffix_array_device(text.data_ptr(), n, sa.data_ptr(), bw.data_ptr(), 0)
    torch.cuda.synchronize()
    s_h = text.cpu().numpy()
    sa_h = sa.cpu().numpy().astype(np.int64)
    del sa
    # suffix order in full: a permutation, adjacent suffixes strictly increasing
    inv = np.full(n + 1, -1, np.int64)
    inv[sa_h] = np.arange(n)
    assert (inv[:n] >= 0).all(), "not a permutation"
    a_, b_ = sa_h[:-1], sa_h[1:]
    assert ((s_h[a_] < s_h[b_]) | ((s_h[a_] == s_h[b_]) & (inv[a_ + 1] < inv[b_ + 1]))).all(), "suffix order"
    del inv, a_, b_
    bw_h = bw.cpu().numpy()
    assert np.array_equal(bw_h, oracle.bwt(s_h, sa_h)), "BWT rule"
    del sa_h, bw
    codes, sigma = oracle.remap_alphabet(bw_h)
    assert sigma == 5
    fm = wtg.FMIndex(codes, sigma)
    _compare_tree(oracle, fm.tree, codes, 3, 1 << 3)
    # backward-search counts of patterns copied from the text
    tcodes, _ = oracle.remap_alphabet(s_h)
    rng = np.random.default_rng(109)
    pats = []
    for _ in range(1 << 14):
        m = int(rng.integers(8, 33))
        i = int(rng.integers(0, n - m))
        pats.append(tcodes[i:i + m])
    pat, off = wtg.FMIndex.pack(pats)
    w, _ = oracle.wt_build(codes, 3, tail=True)
    rt = oracle.rank_build(w, n * 3)
    exp = oracle.fm_count(w, rt, n, 3, fm.C, pat, off)
    got = fm.count(pat, off)
    assert np.array_equal(got, exp)
    fm.tree.free()


def test_batch_4096_texts_against_oracle(wtg, oracle):
    rng = np.random.default_rng(113)
    lengths = np.floor(2.0 ** rng.uniform(10, 20, 4096)).astype(np.uint64)
    concat = rng.integers(0, 4, int(lengths.sum()), dtype=np.uint8)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    b = wtg.Batch(lengths, 2, wtg.ALL)
    b.load(concat)
    b.run()
    b.sync()
    for t in range(lengths.size):
        s = concat[offs[t]:offs[t + 1]]
        n = s.size
        w, _ = oracle.wt_build(s, 2, tail=True)
        assert np.array_equal(b.bits(t), w[:-1]), t
        assert np.array_equal(b.rank_table(t), oracle.rank_build(w, 2 * n)), t
        for t_b in (0, 1):
            o, g = oracle.Select(w, 2 * n, t_b), b.select_tables(t, t_b)
            assert (g.size, g.arg_cnt, g.logn, g.logn4, g.nsb, g.has_long, g.sb_nwords, g.pool_nwords) == \
                   (o.size, o.arg_cnt, o.logn, o.logn4, o.nsb, o.has_long, o.sb_nwords, o.pool_nwords), (t, t_b)
            assert np.array_equal(g.sb_words, o.sb_words), (t, t_b)
            assert np.array_equal(g.desc, o.desc), (t, t_b)
            assert np.array_equal(g.pool, o.pool), (t, t_b)
    b.free()
