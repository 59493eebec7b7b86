"""The reference-shaped C++ interface (host/wtg_reference_api.hpp): WT() with
levelWT's signature and ownership, wt_int, rank_support_v and
select_support_mcl over libwtg.  CPU: the header compiles for the symbol /
index widths the reference builds (-DINT, -DLONG).  GPU: a C++ program using
it matches the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import datagen
from conftest import PKG, ROOT
from helpers import words_with_tail

SRC = os.path.join(ROOT, "tests", "cpp", "wt_api_check.cpp")
VARIANTS = {"u8": [], "int": ["-DINT"], "int_long": ["-DINT", "-DLONG"]}


def _gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("g++ not found")
    return g


@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_header_compiles(variant):
    subprocess.run([_gxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", *VARIANTS[variant], SRC],
                   check=True)


@pytest.mark.gpu
@pytest.mark.parametrize("variant,kind,n", [("u8", "zipf", 100003), ("int", "exp", 65537),
                                            ("int_long", "exp", 4097)])
def test_cpp_program_matches_oracle(wtg, oracle, tmp_path, variant, kind, n):
    lib_dir = os.path.dirname(wtg.lib()._name)
    exe = str(tmp_path / "wt_api_check")
    subprocess.run([_gxx(), "-std=c++17", "-O2", *VARIANTS[variant], SRC, "-o", exe, f"-L{lib_dir}", "-lwtg",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    sym = datagen.zipf_bytes(n, seed=5) if kind == "zipf" else datagen.exp_u32(n, seed=5)
    sym, sigma = oracle.remap_alphabet(sym)
    sym_t = {"u8": np.uint8, "int": np.uint32, "int_long": np.uint64}[variant]
    if variant == "u8":
        assert sigma <= 256
    sym.astype(sym_t).tofile(tmp_path / "s.bin")
    subprocess.run([exe, str(tmp_path / "s.bin"), str(n), str(sigma), str(tmp_path / "o.bin")], check=True)

    L = oracle.levels_for_sigma(sigma)
    ob, on = oracle.wt_build(sym, L, n_nodes=2 * sigma)
    w = words_with_tail(ob)
    orank = oracle.rank_build(w, n * L)
    ib = 8 if variant == "int_long" else 4
    raw = np.fromfile(tmp_path / "o.bin", dtype=np.uint8)
    nb = 2 * sigma * 5 * ib
    nodes = raw[:nb].view(np.uint32 if ib == 4 else np.uint64).reshape(-1, 5)
    rest = raw[nb:].view(np.uint64)
    bits, rank, checks = rest[:ob.size], rest[ob.size:ob.size + orank.size], rest[ob.size + orank.size:]
    exp_nodes = on.astype(np.uint32) if ib == 4 else on
    if ib == 4:
        exp_nodes[on == np.uint64(0xFFFFFFFFFFFFFFFF)] = 0xFFFFFFFF
    assert np.array_equal(nodes, exp_nodes.reshape(-1, 5))
    assert np.array_equal(bits, ob)
    assert np.array_equal(rank, orank)
    assert checks[0] == 0 and checks[1] == 0
    assert checks[2] == int(np.unpackbits(ob.view(np.uint8)).sum())
    # range queries (the layout the program's header states)
    rq = checks[3:]
    assert rq.size == 64 * 9 + 4
    s1, s0 = oracle.Select(w, n * L, 1), oracle.Select(w, n * L, 0)
    for q in range(64):
        i = q * n // 64
        j = min(n, i + n // 8 + 1)
        c = int(sym[i]) if i < n else 0
        row = rq[9 * q:9 * q + 9]
        assert list(row[:3]) == list(oracle.wt_lex_count(w, orank, n, L, [i], [j], [c])[0])
        assert list(row[3:5]) == list(oracle.wt_lex_smaller_count(w, orank, n, L, [i], [c])[0])
        p, _ = oracle.wt_range_report(w, orank, s1, s0, n, L, i, j - 1, c // 2, c)
        assert row[5] == p.size and row[6] == int(p.sum())
        cs, _, _ = oracle.wt_interval_symbols(w, orank, n, L, i, j)
        assert row[7] == cs.size and row[8] == int(cs.sum())
    left, _ = oracle.wt_expand(w, orank, n, [0, n, 0, 0])
    assert rq[-4] == 0 and rq[-3] == 1 and rq[-2] == 1 and rq[-1] == 0 and left[2] == 1
    # sdsl streams written by store_to_file
    out = str(tmp_path / "o.bin")
    assert np.array_equal(np.fromfile(out + ".wt_int", dtype=np.uint8), oracle.serialize_wt_int(sym, L))
    assert np.array_equal(np.fromfile(out + ".rank", dtype=np.uint8), oracle.serialize_rank(orank))
    assert np.array_equal(np.fromfile(out + ".sel1", dtype=np.uint8), oracle.serialize_select(s1))
