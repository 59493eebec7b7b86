"""Huffman-shaped wavelet tree on the GPU (sdsl::wt_huff<>, the reference
FM-index's tree): bitvector, node layout and ranks, codes, rank_support_v and
both select_support_mcl structures bit-exact against the reference's own
wt_huff (golden fixtures) and against the oracle on seeded texts; access,
rank, select and inverse_select against both; FM-index counts over the
Huffman tree of a BWT against the oracle and naive counting."""
import numpy as np
import pytest

import datagen
from test_oracle_huff import HUFF, _ids, _ref_nodes

pytestmark = pytest.mark.gpu


def _compare_structure(t, o):
    """GPU tree t against an oracle.HuffOracle o."""
    assert (t.n, t.sigma, t.size) == (o.n, o.shape.sigma, o.shape.bv_size)
    assert np.array_equal(t.bits(), o.words[:-1])
    nodes, leaves, paths = t.tree()
    nd = nodes.astype(np.int64)
    nd[nd == 0xFFFF] = -1
    assert np.array_equal(nd[:, 0], o.shape.nodes[:, 0])
    assert np.array_equal(nd[:, 2:5], o.shape.nodes[:, 3:6])
    assert np.array_equal(nodes[:, 1], o.node_rank)
    lv = leaves.astype(np.int64)
    lv[lv == 0xFFFF] = -1
    assert np.array_equal(lv, o.shape.leaf)
    assert np.array_equal(paths & np.uint64((1 << 56) - 1), o.shape.path)
    assert np.array_equal((paths >> np.uint64(56)).astype(np.int64), o.shape.plen)
    assert np.array_equal(t.rank_table(), o.rank_tbl)
    for t_b in (0, 1):
        g, s = t.select_tables(t_b), o.sel[t_b]
        assert (g.arg_cnt, g.logn, g.nsb, g.has_long) == (s.arg_cnt, s.logn, s.nsb, s.has_long)
        assert np.array_equal(g.sb_words, s.sb_words)
        assert np.array_equal(g.desc, s.desc)
        assert np.array_equal(g.pool, s.pool)


@pytest.mark.parametrize("path", HUFF, ids=_ids())
def test_matches_reference_golden(wtg, path):
    g = np.load(path)
    t = wtg.HuffmanTree(g["text"])
    assert (t.sigma, t.size) == (int(g["sigma"]), int(g["size"]))
    assert np.array_equal(t.bits(), g["words"])
    nodes, leaves, paths = t.tree()
    assert np.array_equal(nodes, g["nodes"])
    assert np.array_equal(leaves, g["leaf"]) and np.array_equal(paths, g["path"])
    assert np.array_equal(t.rank_table(), g["rank"])
    for t_b in (0, 1):
        s = t.select_tables(t_b)
        assert [s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long, s.sb_nwords, s.pool_nwords] == \
               [int(x) for x in g[f"sel{t_b}_info"]]
        assert np.array_equal(s.sb_words, g[f"sel{t_b}_sb"])
        assert np.array_equal(s.desc, g[f"sel{t_b}_desc"])
        assert np.array_equal(s.pool, g[f"sel{t_b}_pool"])
    assert np.array_equal(t.access(g["acc_i"]), g["acc"])
    assert np.array_equal(t.rank(g["rank_i"], g["rank_c"]), g["rank_ans"])
    assert np.array_equal(t.select(g["sel_i"], g["sel_c"]), g["sel_ans"])
    t.free()


def _text(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "zipf":
        return datagen.zipf_bytes(n, seed=seed)
    if kind == "dna":
        return datagen.dna_markov(n, seed=seed)
    if kind == "bytes":
        return rng.integers(0, 256, n).astype(np.uint8)
    if kind == "skew":  # geometric counts: long codes
        return np.minimum(rng.geometric(0.35, n), 40).astype(np.uint8)
    if kind == "one":
        return np.full(n, 9, dtype=np.uint8)
    return rng.integers(0, 2, n).astype(np.uint8)


@pytest.mark.parametrize("kind,n", [("zipf", 1 << 20), ("dna", 300007), ("bytes", 100000), ("skew", 200001),
                                    ("one", 1000), ("two", 70001), ("zipf", 1), ("bytes", 513), ("zipf", 0)])
def test_matches_oracle(wtg, oracle, kind, n):
    text = _text(kind, n, n + 5)
    t = wtg.HuffmanTree(text)
    if n == 0:
        assert (t.n, t.sigma, t.size) == (0, 0, 0)
        return
    o = oracle.HuffOracle(text)
    _compare_structure(t, o)
    rng = np.random.default_rng(n)
    qi = rng.integers(0, n, 3000).astype(np.uint64)
    assert np.array_equal(t.access(qi), text[qi.astype(np.int64)].astype(np.uint64))
    r, c = t.inverse_select(qi)
    assert np.array_equal(c, text[qi.astype(np.int64)].astype(np.uint64))
    for k in range(0, 3000, 300):
        i = int(qi[k])
        assert int(r[k]) == int(np.count_nonzero(text[:i] == text[i]))
    ri = rng.integers(0, n + 1, 3000).astype(np.uint64)
    rc = np.concatenate([text[rng.integers(0, n, 2900)], rng.integers(0, 256, 100).astype(np.uint8)]).astype(np.uint64)
    exp = np.array([o.rank(int(i), int(cc)) for i, cc in zip(ri, rc)], dtype=np.uint64)
    assert np.array_equal(t.rank(ri, rc), exp)
    sc = text[rng.integers(0, n, 1000)].astype(np.uint64)
    occ = {int(x): int(np.count_nonzero(text == x)) for x in np.unique(sc)}
    si = np.array([rng.integers(1, occ[int(x)] + 1) for x in sc], dtype=np.uint64)
    got = t.select(si, sc)
    assert np.array_equal(got, np.array([o.select(int(i), int(cc)) for i, cc in zip(si, sc)], dtype=np.uint64))
    assert np.all(text[got.astype(np.int64)] == sc)
    t.free()


def test_fm_index_counts(wtg, oracle):
    text = datagen.dna_markov(200000, seed=41)
    text = np.concatenate([text, np.frombuffer(b"$", np.uint8)])  # a unique smallest terminator
    b = oracle.bwt(text, oracle.suffix_array(text))
    t = wtg.HuffmanTree(b)
    counts = np.bincount(text, minlength=256).astype(np.uint64)
    C = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
    rng = np.random.default_rng(3)
    pats = [text[i:i + m] for i, m in zip(rng.integers(0, text.size - 40, 400), rng.integers(1, 33, 400))]
    pats += [np.frombuffer(b"NNNNACGT", np.uint8), np.frombuffer(b"zz", np.uint8), np.zeros(0, np.uint8)]
    off = np.concatenate([[0], np.cumsum([p.size for p in pats])]).astype(np.uint64)
    pat = np.concatenate(pats)
    got = t.fm_count(C, pat, off)
    s = text.tobytes()
    for q, p in enumerate(pats):
        if p.size == 0:
            assert got[q] == text.size
            continue
        pb = p.tobytes()
        exp, k = 0, s.find(pb)
        while k >= 0:
            exp += 1
            k = s.find(pb, k + 1)
        assert got[q] == exp, q
    t.free()


def test_fm_count_device_matches_host(wtg, oracle):
    torch = pytest.importorskip("torch")
    text = datagen.dna_markov(100000, seed=43)
    text = np.concatenate([text, np.frombuffer(b"$", np.uint8)])
    b = oracle.bwt(text, oracle.suffix_array(text))
    t = wtg.HuffmanTree(b)
    counts = np.bincount(text, minlength=256).astype(np.uint64)
    C = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
    rng = np.random.default_rng(5)
    pats = [text[i:i + m] for i, m in zip(rng.integers(0, text.size - 40, 300), rng.integers(1, 33, 300))]
    off = np.concatenate([[0], np.cumsum([p.size for p in pats])]).astype(np.uint64)
    pat = np.concatenate(pats)
    host = t.fm_count(C, pat, off)
    dev = torch.device("cuda")
    dC = torch.from_numpy(C.view(np.int64)).to(dev)
    dpat = torch.from_numpy(pat).to(dev)
    doff = torch.from_numpy(off.view(np.int64)).to(dev)
    dout = torch.empty(len(pats), dtype=torch.int64, device=dev)
    t.fm_count_device(dC.data_ptr(), dpat.data_ptr(), doff.data_ptr(), len(pats), dout.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy().view(np.uint64), host)
    t.free()
