"""Generates tests/golden/huff/*.npz from the reference's own Huffman-shaped
wavelet tree.

Runs wt_huff/wt_huff_par.hpp (sdsl::wt_huff = wt_pc with the Huffman shape,
built by wt_huff/wt_pc_par.hpp) compiled from the read-only reference checkout
into oracle/_ref/libref_wt_huff.so (`make -C oracle ref`, against the sdsl
stand-in in oracle/sdsl_shim, which restates the breadth-first byte code tree
wt_pc lays its nodes out in).  Per case it stores the text, the concatenated
bitvector, the rank_support_v table, both select_support_mcl structures
(flat layout), the node table (bv_pos, bv_pos_rank, parent, child0, child1;
0xFFFF for none), each byte's leaf and path, and seeded queries with the
reference's answers: access, rank(i, c) and select(i, c).

Usage: python tests/golden/make_golden_huff.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "huff")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300"))

from oracle import oracle as O  # noqa: E402
import datagen  # noqa: E402

NQ = 300


def cases():
    rng = np.random.default_rng(31)
    yield "mississippi", np.frombuffer(b"mississippi", dtype=np.uint8).copy()
    yield "single_7_50", np.full(50, 7, dtype=np.uint8)
    yield "two_symbols_1000", rng.integers(3, 5, 1000).astype(np.uint8)
    yield "dna_markov_20000", datagen.dna_markov(20000, seed=32)
    yield "zipf_bytes_65536", datagen.zipf_bytes(65536, seed=33)
    yield "uniform_bytes_30000", rng.integers(0, 256, 30000).astype(np.uint8)
    # skewed counts: a deep code (Fibonacci-like frequencies)
    fib = [1, 1]
    while len(fib) < 20:
        fib.append(fib[-1] + fib[-2])
    yield "fibonacci_counts", np.repeat(np.arange(20, dtype=np.uint8), fib)[rng.permutation(sum(fib))]


def main():
    O.build(ref=True)
    os.makedirs(OUT, exist_ok=True)
    for name, text in cases():
        R = O.RefWtHuff(text)
        rng = np.random.default_rng(text.size + 7)
        n = text.size
        out = {"text": text, "words": R.words, "rank": R.rank_tbl, "nodes": R.nodes, "leaf": R.leaf, "path": R.path,
               "sigma": np.int64(R.sigma), "size": np.int64(R.size)}
        for t_b in (0, 1):
            info, sb, desc, pool = R.select_tables(t_b)
            out[f"sel{t_b}_info"], out[f"sel{t_b}_sb"], out[f"sel{t_b}_desc"], out[f"sel{t_b}_pool"] = info, sb, desc, pool
        qi = rng.integers(0, n, NQ).astype(np.uint64)
        out["acc_i"] = qi
        out["acc"] = np.array([R.access(i) for i in qi], dtype=np.uint64)
        ri = rng.integers(0, n + 1, NQ).astype(np.uint64)
        rc = np.concatenate([text[rng.integers(0, n, NQ - 20)], rng.integers(0, 256, 20).astype(np.uint8)])
        out["rank_i"], out["rank_c"] = ri, rc.astype(np.uint64)
        out["rank_ans"] = np.array([R.rank(i, c) for i, c in zip(ri, rc)], dtype=np.uint64)
        sc = text[rng.integers(0, n, NQ)]
        occ = {int(c): int(np.count_nonzero(text == c)) for c in np.unique(sc)}
        si = np.array([rng.integers(1, occ[int(c)] + 1) for c in sc], dtype=np.uint64)
        out["sel_i"], out["sel_c"] = si, sc.astype(np.uint64)
        out["sel_ans"] = np.array([R.select(i, c) for i, c in zip(si, sc)], dtype=np.uint64)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
        print(name, n, "sigma", R.sigma, "bits", R.size, "nodes", R.nodes.shape[0])


if __name__ == "__main__":
    main()
