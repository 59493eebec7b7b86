"""FM-index oracle pinned to the reference: the suffix array and BWT equal the
reference's vendored divsufsort and the BWT rule of fm-index/par/WT.C:38-41
(golden vectors, and live when the reference build exists); backward search
counts equal naive occurrence counts on texts with a unique smallest
terminator (without one, the BWT wraps s[n-1] to the front and counts can
differ near that entry -- the GPU reproduces the oracle there too)."""
import glob
import os

import numpy as np
import pytest

import datagen
from helpers import words_with_tail

FM_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fm", "*.npz")))


@pytest.mark.parametrize("path", FM_GOLDEN, ids=[os.path.basename(p)[:-4] for p in FM_GOLDEN])
def test_sa_and_bwt_match_reference_golden(oracle, path):
    g = np.load(path)
    sa = oracle.suffix_array(g["text"])
    assert np.array_equal(sa, g["sa"])
    assert np.array_equal(oracle.bwt(g["text"], sa), g["bwt"])


def test_sa_matches_live_reference(oracle):
    if not oracle.ref_available("divsufsort"):
        pytest.skip("reference build not present")
    rng = np.random.default_rng(5)
    for s in (np.zeros(1, np.uint8), np.frombuffer(b"abracadabra", np.uint8), rng.integers(0, 2, 5000).astype(np.uint8),
              rng.integers(0, 256, 20000).astype(np.uint8), datagen.dna_markov(50000, seed=8)):
        assert np.array_equal(oracle.suffix_array(s), oracle.ref_divsufsort(s).astype(np.int64))


def fm_oracle(oracle, codes, sigma):
    sa = oracle.suffix_array(codes)
    bwt = oracle.bwt(codes, sa)
    L = oracle.levels_for_sigma(sigma)
    bits, _ = oracle.wt_build(bwt, L)
    w = words_with_tail(bits)
    rt = oracle.rank_build(w, bwt.size * L)
    C = np.concatenate([[0], np.cumsum(np.bincount(bwt, minlength=sigma))]).astype(np.uint64)[:sigma]
    return bwt, L, w, rt, C


def naive_count(text, p):
    s, pb = text.tobytes(), np.asarray(p, dtype=np.uint8).tobytes()
    return sum(1 for i in range(len(s) - len(pb) + 1) if s[i:i + len(pb)] == pb)


def test_backward_search_counts_occurrences_with_terminator(oracle):
    rng = np.random.default_rng(1)
    for text in (datagen.dna_markov(8000, seed=3), np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 9000)]):
        codes, sigma = oracle.remap_alphabet(text)
        codes = np.concatenate([codes + 1, [0]]).astype(np.uint8)
        sigma += 1
        bwt, L, w, rt, C = fm_oracle(oracle, codes, sigma)
        pats = [codes[i:i + m] for i, m in zip(rng.integers(0, codes.size - 40, 120), rng.integers(1, 25, 120))]
        pats += [np.array([1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1], np.uint8), np.array([], np.uint8)]
        off = np.zeros(len(pats) + 1, np.uint64)
        off[1:] = np.cumsum([len(p) for p in pats])
        got = oracle.fm_count(w, rt, bwt.size, L, C, np.concatenate(pats).astype(np.uint8), off)
        exp = [naive_count(codes, p) if len(p) else codes.size for p in pats]
        assert list(got) == exp
