"""Generates the FM-index golden vectors under fm/ from the reference itself.

Runs the reference's vendored libdivsufsort (suffixArray/divsufsort, compiled
into oracle/_ref/ by `make -C oracle ref`) on seeded texts and stores the text,
its suffix array and the BWT by the rule of fm-index/par/WT.C:38-41
(bwt[i] = s[SA[i]-1], or s[n-1] where SA[i] == 0) as fm/<name>.npz.

Usage: python tests/golden/make_golden_fm.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300"))

from oracle import oracle as O  # noqa: E402
import datagen  # noqa: E402


def cases():
    rng = np.random.default_rng(77)
    yield "banana", np.frombuffer(b"banana", dtype=np.uint8)
    yield "mississippi", np.frombuffer(b"mississippi", dtype=np.uint8)
    yield "allA_2000", np.full(2000, ord("A"), dtype=np.uint8)
    yield "periodic_ACG_3001", np.resize(np.frombuffer(b"ACG", dtype=np.uint8), 3001)
    yield "dna_markov_40000", datagen.dna_markov(40000, seed=21)
    yield "acgt_uniform_65536", np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, 65536)]


def main():
    O.build(ref=True)
    os.makedirs(os.path.join(HERE, "fm"), exist_ok=True)
    for name, s in cases():
        s = np.ascontiguousarray(s, dtype=np.uint8)
        sa = O.ref_divsufsort(s).astype(np.int64)
        bwt = s[np.where(sa == 0, s.size - 1, sa - 1)]
        np.savez_compressed(os.path.join(HERE, "fm", name + ".npz"), text=s, sa=sa, bwt=bwt)
        print(name, s.size)


if __name__ == "__main__":
    main()
