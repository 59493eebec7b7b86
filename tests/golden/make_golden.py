"""Generates the golden vectors in this directory from the reference itself.

Runs the reference's own builders, compiled from its sources into oracle/_ref/
(`make -C oracle ref`, which needs the read-only reference checkout):
  * WT() of wavelet/levelWT/WT.C (byte symbols, -DINT, -DLONG -DINT) -> the
    level bitvector and the node records;
  * rank_support_v<1> and select_support_mcl<1>/<0> of
    rank/rank_support_v_par.hpp and select/select_support_mcl_par.hpp (built
    against the sdsl stand-in in oracle/sdsl_shim) over that bitvector.
Each case is stored as <name>.npz.  Inputs come from the seeded generators of
the package (datagen.py), remapped to their dense alphabet as the reference's
WTTime.C driver does (levelWT/WTTime.C:80-94) unless sigma is given.

Usage: python tests/golden/make_golden.py
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
    rng = np.random.default_rng(2024)
    yield "zipf_u8_65537", datagen.zipf_bytes(65537, seed=11), None, "levelwt_u8"
    yield "rand_u8_777_s5", rng.integers(0, 5, 777).astype(np.uint8), None, "levelwt_u8"
    yield "allequal_u8_1000", np.full(1000, 7, dtype=np.uint8), None, "levelwt_u8"
    yield "alternating_u8_4096", np.tile(np.array([3, 9], dtype=np.uint8), 2048), None, "levelwt_u8"
    runs = np.repeat(rng.integers(0, 200, 1000).astype(np.uint8), rng.integers(1, 200, 1000))[:100003]
    yield "runs_u8_s200", runs, None, "levelwt_u8"
    yield "dna_u8_20000", datagen.dna_markov(20000, seed=5), None, "levelwt_u8"
    yield "single_u8_1", np.array([42], dtype=np.uint8), None, "levelwt_u8"
    yield "exp_u32_32768_L20", datagen.exp_u32(32768, seed=3), 1 << 20, "levelwt_int"
    yield "rand_u32_70001_s1000", rng.integers(0, 1000, 70001).astype(np.uint32), None, "levelwt_int"
    yield "exp_u64_20000_L20_long", datagen.exp_u32(20000, seed=4).astype(np.uint64), 1 << 20, "levelwt_long_int"


def main():
    O.build(ref=True)
    for name, sym, sigma, variant in cases():
        if sigma is None:
            sym, sigma = O.remap_alphabet(sym)
        levels = O.levels_for_sigma(sigma)
        bits, nodes = O.ref_wt(sym, sigma, variant)
        none = 0xFFFFFFFF if nodes.dtype == np.uint32 else 0xFFFFFFFFFFFFFFFF
        reach = np.array(O.reachable_nodes(nodes, none), dtype=np.int64)
        size = sym.size * levels
        words = np.concatenate([bits, np.zeros(1, np.uint64)])
        rank = O.ref_rank_build(words, size)
        out = dict(sym=sym, sigma=np.uint64(sigma), levels=np.int64(levels), bits=bits,
                   node_ids=reach, nodes=nodes[reach], node_none=np.uint64(none), rank=rank)
        for t_b in (0, 1):
            s = O.RefSelect(words, size, t_b)
            out[f"sel{t_b}_info"] = np.array([s.size, s.arg_cnt, s.logn, s.logn4, s.nsb, s.has_long,
                                              s.sb_nwords, s.pool_nwords], dtype=np.uint64)
            out[f"sel{t_b}_sb"] = s.sb_words
            out[f"sel{t_b}_desc"] = s.desc
            out[f"sel{t_b}_pool"] = s.pool
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, sym.dtype, sym.size, "sigma", sigma, "levels", levels, "nodes", reach.size)


if __name__ == "__main__":
    main()
