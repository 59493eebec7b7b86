"""Shared helpers for the tests (expected-value construction uses the oracle)."""
import glob
import os

import numpy as np

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))
NONE64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def golden_ids():
    return [os.path.basename(p)[:-4] for p in GOLDEN]


def ref_nodes_u64(g):
    """Golden node records widened to u64 with UINT64_MAX for absent links."""
    ref = g["nodes"].astype(np.uint64)
    ref[g["nodes"] == g["node_none"]] = NONE64
    return ref


def words_with_tail(bits):
    return np.concatenate([np.asarray(bits, dtype=np.uint64), np.zeros(1, np.uint64)])


def unpack_bits(words, size):
    b = np.unpackbits(np.asarray(words, dtype=np.uint64).view(np.uint8), bitorder="little")
    return b[:size].astype(np.uint8)
