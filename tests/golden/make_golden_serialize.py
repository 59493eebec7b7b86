"""Generates tests/golden/serialize/*.npz: sdsl serialize() byte streams
written by the reference's own classes.

The reference's wt_int (wt_int/wt_int_par.hpp:887-899), rank_support_v
(rank/rank_support_v_par.hpp:154-164) and select_support_mcl
(select/select_support_mcl_par.hpp:644-681) are compiled from the read-only
reference checkout into oracle/_ref/ (`make -C oracle ref`) against the sdsl
stand-in in oracle/sdsl_shim, whose int_vector writes sdsl's format (size in
bits as u64, width byte for run-time widths, ceil(bits/64) words).  Per case
the input and the reference's stream are stored.

Usage: python tests/golden/make_golden_serialize.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "serialize")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300"))

from oracle import oracle as O  # noqa: E402
import datagen  # noqa: E402


def tree_cases():
    rng = np.random.default_rng(91)
    yield "wt_empty_u8_L3", np.zeros(0, dtype=np.uint8), 3
    yield "wt_pi_u8_L0", np.array([3, 1, 4, 1, 5, 9, 2, 6, 5, 3], dtype=np.uint8), 0
    yield "wt_exp_u32_L20_70001", datagen.exp_u32(70001, seed=92), 20
    yield "wt_zipf_u8_L8_150001", datagen.zipf_bytes(150001, seed=93), 8
    yield "wt_rand_u16_L12_30001", rng.integers(0, 3000, 30001).astype(np.uint16), 12


def bv_cases():
    yield "bv_sparse_1048576", 1 << 20, 0.0005
    yield "bv_dense_1048653", (1 << 20) + 77, 0.3
    yield "bv_slow_99999", 99999, 0.01
    yield "bv_empty_0", 0, 0.5


def main():
    O.build(ref=True)
    os.makedirs(OUT, exist_ok=True)
    for name, sym, L in tree_cases():
        R = O.RefWtInt(sym, L)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), sym=sym, levels=np.int64(L), stream=R.serialize())
        print(name, R.serialize().size)
    for name, size, dens in bv_cases():
        words = datagen.random_bits(size, dens, seed=size + 5)
        w = np.concatenate([words, np.zeros(1, np.uint64)])
        out = {"words": words, "size": np.int64(size), "rank": O.ref_rank_serialize(w, size)}
        for t_b in (0, 1):
            out[f"sel{t_b}"] = O.RefSelect(w, size, t_b).serialize()
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
        print(name, {k: v.size for k, v in out.items()})


if __name__ == "__main__":
    main()
