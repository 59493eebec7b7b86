"""Generates tests/golden/wt_int/*.npz from the reference's own sdsl::wt_int.

Runs wt_int/wt_int_par.hpp -- its constructor and its query members --
compiled from the read-only reference checkout into
oracle/_ref/libref_wt_int.so (`make -C oracle ref`, against the sdsl
stand-in in oracle/sdsl_shim).  Per case it stores the input, the tree bits
and, for seeded queries, the reference's answers of operator[], rank,
select, inverse_select, lex_count, lex_smaller_count, range_search_2d (count
and reported points), interval_symbols, expand(v) and expand(v, ranges).
Variable-length answers are stored flat with per-query offsets.

Usage: python tests/golden/make_golden_wt_int.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "wt_int")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300"))

from oracle import oracle as O  # noqa: E402
import datagen  # noqa: E402

NQ = 400


def cases():
    rng = np.random.default_rng(77)
    yield "rand_u8_L5_1000", rng.integers(0, 32, 1000).astype(np.uint8), 5
    yield "zipf_u8_L8_20011", datagen.zipf_bytes(20011, seed=8), 8
    yield "rand_u16_L12_30001", rng.integers(0, 3000, 30001).astype(np.uint16), 12
    yield "exp_u32_L20_7001", datagen.exp_u32(7001, seed=21), 20
    yield "allsame_u8_L3_777", np.full(777, 5, dtype=np.uint8), 3
    yield "tiny_u8_L3_5", np.array([4, 1, 7, 1, 0], dtype=np.uint8), 3
    yield "sparse_u32_L24_4097", (rng.integers(0, 4, 4097) * 4000003).astype(np.uint32), 24


def inner_nodes(R, n, L, rng, count):
    """(offset, size, level, sym) of inner nodes on random root-to-leaf walks."""
    out = []
    while len(out) < count:
        v = np.array([0, n, 0, 0], dtype=np.uint64)
        for _ in range(L):
            out.append(v.copy())
            left, right = R.expand(v)
            v = left if (rng.integers(0, 2) == 0 and left[1] > 0) or right[1] == 0 else right
    return np.array(out[:count], dtype=np.uint64)


def main():
    O.build(ref=True)
    os.makedirs(OUT, exist_ok=True)
    for name, sym, L in cases():
        rng = np.random.default_rng(sym.size * 31 + L)
        n = sym.size
        R = O.RefWtInt(sym, L)
        g = dict(sym=sym, levels=np.int64(L), bits=R.bits, sigma=np.uint64(R.sigma))
        top = (1 << L) + 3
        # point queries
        idx = rng.integers(0, n, NQ).astype(np.uint64)
        g["access_i"] = idx
        g["access"] = np.array([R.access(i) for i in idx], dtype=np.uint64)
        inv = np.array([R.inverse_select(i) for i in idx], dtype=np.uint64)
        g["inv_rank"], g["inv_sym"] = inv[:, 0], inv[:, 1]
        ri = rng.integers(0, n + 1, NQ).astype(np.uint64)
        rc = np.where(rng.integers(0, 4, NQ) == 0, rng.integers(0, top, NQ), sym[rng.integers(0, n, NQ)])
        g["rank_i"], g["rank_c"] = ri, rc.astype(np.uint64)
        g["rank"] = np.array([R.rank(i, c) for i, c in zip(ri, rc)], dtype=np.uint64)
        sc = sym[rng.integers(0, n, NQ)].astype(np.uint64)
        occ = np.array([R.rank(n, c) for c in sc], dtype=np.int64)
        si = np.array([rng.integers(1, o + 2) for o in occ], dtype=np.uint64)  # some past the count
        g["select_i"], g["select_c"] = si, sc
        g["select"] = np.array([R.select(i, c) for i, c in zip(si, sc)], dtype=np.uint64)
        # lex_count / lex_smaller_count
        i = rng.integers(0, n + 1, NQ)
        j = np.minimum(n, i + rng.integers(0, n + 1, NQ) // rng.integers(1, 64, NQ))
        c = np.where(rng.integers(0, 3, NQ) == 0, rng.integers(0, top, NQ), sym[rng.integers(0, n, NQ)])
        g["lex_i"], g["lex_j"], g["lex_c"] = i.astype(np.uint64), j.astype(np.uint64), c.astype(np.uint64)
        g["lex_count"] = np.array([R.lex_count(a, b, x) for a, b, x in zip(i, j, c)], dtype=np.uint64)
        g["lex_smaller"] = np.array([R.lex_smaller_count(a, x) for a, x in zip(i, c)], dtype=np.uint64)
        # range_search_2d
        lb = rng.integers(0, n, NQ)
        rb = np.minimum(n - 1, lb + rng.integers(0, n, NQ) // rng.integers(1, 64, NQ))
        lb[:8] = rb[:8] + 1  # empty position ranges
        lb[:4] = np.minimum(lb[:4], n - 1)
        rb[:4] = lb[:4] - 1 if n > 1 else rb[:4]
        vlb = rng.integers(0, top, NQ)
        vrb = vlb + rng.integers(0, 1 << L, NQ) // rng.integers(1, 16, NQ)
        vlb[8:40] = 0
        vrb[40:60] = (1 << L) + 100  # clamped to 2^L
        vlb[60:70] = vrb[60:70] + 1  # empty value ranges
        g["r2d_lb"], g["r2d_rb"] = lb.astype(np.uint64), rb.astype(np.uint64)
        g["r2d_vlb"], g["r2d_vrb"] = vlb.astype(np.uint64), vrb.astype(np.uint64)
        cnts, pos, val = [], [], []
        for q in range(NQ):
            cnt, p, v = R.range_search_2d(lb[q], rb[q], vlb[q], vrb[q], report=q < NQ // 2)
            cnts.append(cnt)
            if q < NQ // 2:
                pos.append(p)
                val.append(v)
        g["r2d_count"] = np.array(cnts, dtype=np.uint64)
        g["r2d_report_q"] = np.int64(NQ // 2)  # queries 0..NQ/2-1 carry reported points
        g["r2d_pos"] = np.concatenate(pos).astype(np.uint64)
        g["r2d_val"] = np.concatenate(val).astype(np.uint64)
        # interval_symbols
        i = rng.integers(0, n + 1, NQ)
        j = np.minimum(n, i + rng.integers(0, n + 1, NQ) // rng.integers(1, 256, NQ))
        j[:20] = i[:20]
        j[20:40] = np.minimum(n, i[20:40] + 1)
        g["isym_i"], g["isym_j"] = i.astype(np.uint64), j.astype(np.uint64)
        ks, cs, ris, rjs = [], [], [], []
        for a, b in zip(i, j):
            x, y, z = R.interval_symbols(a, b)
            ks.append(x.size)
            cs.append(x)
            ris.append(y)
            rjs.append(z)
        g["isym_k"] = np.array(ks, dtype=np.uint64)
        g["isym_cs"] = np.concatenate(cs).astype(np.uint64)
        g["isym_ri"] = np.concatenate(ris).astype(np.uint64)
        g["isym_rj"] = np.concatenate(rjs).astype(np.uint64)
        # expand(v) and expand(v, ranges)
        nodes = inner_nodes(R, n, L, rng, 64)
        g["exp_nodes"] = nodes
        ch = [R.expand(v) for v in nodes]
        g["exp_left"] = np.array([a for a, _ in ch], dtype=np.uint64)
        g["exp_right"] = np.array([b for _, b in ch], dtype=np.uint64)
        v = nodes[int(np.argmax(nodes[:, 1]))] if L > 1 else nodes[0]
        sz = int(v[1])
        s = rng.integers(0, max(sz, 1), 200)
        e = np.minimum(sz - 1, s + rng.integers(0, sz + 1, 200) // rng.integers(1, 16, 200))
        e[:10] = s[:10] - 1  # empty ranges (e = s - 1, wrapping at s = 0)
        ranges = np.stack([s, e], axis=1).astype(np.int64).view(np.uint64)
        left, right = R.expand_ranges(v, ranges)
        g["expr_node"], g["expr_ranges"], g["expr_left"], g["expr_right"] = v, ranges, left, right
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **g)
        print(name, sym.dtype, n, "L", L, "sigma", R.sigma, "points", g["r2d_pos"].size, "symbols",
              g["isym_cs"].size)


if __name__ == "__main__":
    main()
