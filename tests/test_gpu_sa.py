"""Suffix array and BWT on the GPU (fm-index/par/WT.C:33-41): identical to
the reference's own divsufsort (golden vectors in tests/golden/fm/) and to the
oracle's suffix array on seeded texts of every alphabet size and on the
repetitive texts that need many doubling rounds; at 2^24 symbols the order is
checked in full through the inverse array."""
import glob
import os

import numpy as np
import pytest

import datagen

pytestmark = pytest.mark.gpu

FM = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fm", "*.npz")))


@pytest.mark.parametrize("path", FM, ids=[os.path.basename(p)[:-4] for p in FM])
def test_matches_reference_divsufsort(wtg, path):
    g = np.load(path)
    b, sa = wtg.bwt(g["text"], with_sa=True)
    assert np.array_equal(sa, g["sa"].astype(np.int32))
    assert np.array_equal(b, g["bwt"])
    assert np.array_equal(wtg.suffix_array(g["text"]), g["sa"].astype(np.int32))


def _texts():
    rng = np.random.default_rng(7)
    yield "one", np.array([42], np.uint8)
    yield "two_eq", np.array([5, 5], np.uint8)
    yield "two", np.array([9, 3], np.uint8)
    yield "zeros_4097", np.zeros(4097, np.uint8)
    yield "binary_100003", rng.integers(0, 2, 100003).astype(np.uint8)
    yield "dna_4096", rng.choice(np.frombuffer(b"ACGT", np.uint8), 4096)
    yield "dna_markov_300001", datagen.dna_markov(300001, seed=3)
    yield "bytes_65537", rng.integers(0, 256, 65537).astype(np.uint8)
    yield "bytes_with_zero_255", rng.integers(0, 255, 70000).astype(np.uint8)
    yield "periodic_abc_20000", np.tile(np.frombuffer(b"abc", np.uint8), 6667)[:20000]
    yield "runs_50000", np.repeat(rng.integers(0, 4, 600).astype(np.uint8), rng.integers(1, 160, 600))[:50000]
    yield "fibonacci_46368", _fib(46368)


def _fib(n):
    a, b = b"a", b"ab"
    while len(b) < n:
        a, b = b, b + a
    return np.frombuffer(b[:n], np.uint8).copy()


@pytest.mark.parametrize("name,text", list(_texts()), ids=[t[0] for t in _texts()])
def test_matches_oracle(wtg, oracle, name, text):
    b, sa = wtg.bwt(text, with_sa=True)
    exp = oracle.suffix_array(text)
    assert np.array_equal(sa.astype(np.int64), exp)
    assert np.array_equal(b, oracle.bwt(text, exp))


def test_empty_text(wtg):
    assert wtg.suffix_array(np.zeros(0, np.uint8)).size == 0
    assert wtg.bwt(np.zeros(0, np.uint8)).size == 0


def test_order_at_scale(wtg):
    """2^24 symbols of an order-2 DNA Markov text with N runs: SA is a
    permutation and every adjacent pair is in suffix order (first symbols,
    then the inverse array one position on)."""
    n = 1 << 24
    s = datagen.dna_markov(n, seed=11)
    sa = wtg.suffix_array(s).astype(np.int64)
    inv = np.empty(n + 1, np.int64)
    inv[sa] = np.arange(n)
    inv[n] = -1  # the empty suffix sorts first
    assert np.array_equal(np.sort(sa), np.arange(n))
    a, b = sa[:-1], sa[1:]
    ok = (s[a] < s[b]) | ((s[a] == s[b]) & (inv[a + 1] < inv[b + 1]))
    assert bool(ok.all())


def test_fm_index_from_text_counts(wtg, oracle):
    s = datagen.dna_markov(200003, seed=5)
    fm, code = wtg.FMIndex.from_text(s)
    rng = np.random.default_rng(2)
    pats = []
    for _ in range(300):
        p = int(rng.integers(0, s.size - 40))
        pats.append(code[s[p:p + int(rng.integers(1, 30))]].astype(np.uint8))
    pat, off = wtg.FMIndex.pack(pats)
    got = fm.count(pat, off)
    sa = oracle.suffix_array(s)
    bw = oracle.bwt(s, sa)
    bits, _ = oracle.wt_build(code[bw].astype(np.uint8), oracle.levels_for_sigma(fm.sigma))
    from helpers import words_with_tail
    w = words_with_tail(bits)
    rt = oracle.rank_build(w, s.size * oracle.levels_for_sigma(fm.sigma))
    exp = oracle.fm_count(w, rt, s.size, oracle.levels_for_sigma(fm.sigma), fm.C, pat, off)
    assert np.array_equal(got, exp)


def test_device_entry_point(wtg):
    import torch
    s = datagen.dna_markov(1 << 20, seed=9)
    d = torch.from_numpy(s).cuda()
    sa = torch.empty(s.size, dtype=torch.int32, device="cuda")
    bw = torch.empty(s.size, dtype=torch.uint8, device="cuda")
    rounds = wtg.suffix_array_device(d.data_ptr(), s.size, sa.data_ptr(), bw.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    assert rounds >= 1
    b2, sa2 = wtg.bwt(s, with_sa=True)
    assert np.array_equal(sa.cpu().numpy(), sa2) and np.array_equal(bw.cpu().numpy(), b2)
