"""FM-index counting on the GPU: backward search over the GPU wavelet tree of
the BWT equals the oracle's backward search (reference SA and BWT from the
golden vectors, plus seeded DNA-like texts), through the host and device
entry points; with a unique terminator the counts equal naive occurrence
counts."""
import glob
import os

import numpy as np
import pytest

import datagen
from test_oracle_fm import fm_oracle, naive_count

pytestmark = pytest.mark.gpu

FM_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fm", "*.npz")))


def _patterns(rng, codes, sigma, count):
    pats = []
    for _ in range(count):
        m = int(rng.integers(1, 33))
        i = int(rng.integers(0, max(1, codes.size - m + 1)))
        pats.append(codes[i:i + m])
    # absent and odd patterns: random codes, a code outside the alphabet, empty
    pats += [rng.integers(0, sigma, 20).astype(np.uint8) for _ in range(8)]
    pats += [np.array([sigma], np.uint8) if sigma < 256 else np.array([0], np.uint8), np.array([], np.uint8)]
    return pats


def _check(wtg, oracle, codes, sigma, npat, seed):
    bwt, L, w, rt, C = fm_oracle(oracle, codes, sigma)
    fm = wtg.FMIndex(bwt, sigma)
    assert np.array_equal(fm.C, C)
    rng = np.random.default_rng(seed)
    pat, off = wtg.FMIndex.pack(_patterns(rng, codes, sigma, npat))
    exp = oracle.fm_count(w, rt, bwt.size, L, C, pat, off)
    got = fm.count(pat, off)
    assert np.array_equal(got, exp)
    return fm, pat, off, exp


@pytest.mark.parametrize("path", FM_GOLDEN, ids=[os.path.basename(p)[:-4] for p in FM_GOLDEN])
def test_counts_on_reference_bwt_match_oracle(wtg, oracle, path):
    g = np.load(path)
    codes, sigma = oracle.remap_alphabet(g["text"])
    bwt_ref, _ = oracle.remap_alphabet(g["bwt"])
    sa = oracle.suffix_array(codes)
    assert np.array_equal(oracle.bwt(codes, sa), bwt_ref)  # the reference's BWT, in codes
    _check(wtg, oracle, codes, sigma, 3000, seed=codes.size)


@pytest.mark.parametrize("n", [1 << 20, (1 << 18) + 3])
def test_counts_on_dna_text(wtg, oracle, n):
    codes, sigma = oracle.remap_alphabet(datagen.dna_markov(n, seed=n))
    _check(wtg, oracle, codes, sigma, 1 << 16, seed=1)


def test_terminated_text_counts_are_occurrences(wtg, oracle):
    codes, sigma = oracle.remap_alphabet(datagen.dna_markov(6000, seed=4))
    codes = np.concatenate([codes + 1, [0]]).astype(np.uint8)
    fm, pat, off, got = _check(wtg, oracle, codes, sigma + 1, 200, seed=2)
    for p in range(off.size - 1):
        a, b = int(off[p]), int(off[p + 1])
        exp = naive_count(codes, pat[a:b]) if b > a else codes.size
        assert got[p] == exp


def test_device_entry_point(wtg, oracle):
    import torch
    codes, sigma = oracle.remap_alphabet(datagen.dna_markov(1 << 16, seed=6))
    fm, pat, off, exp = _check(wtg, oracle, codes, sigma, 4000, seed=3)
    dC = torch.from_numpy(fm.C.view(np.int64)).cuda()
    dpat = torch.from_numpy(pat).cuda()
    doff = torch.from_numpy(off.view(np.int64)).cuda()
    dout = torch.empty(off.size - 1, dtype=torch.int64, device="cuda")
    fm.count_device(dC.data_ptr(), dpat.data_ptr(), doff.data_ptr(), off.size - 1, dout.data_ptr(),
                    torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy().view(np.uint64), exp)
