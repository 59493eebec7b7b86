"""A tree past 2^31 symbols (3 * 2^30 + 37 byte symbols, 3 levels, n not a
multiple of 32): positions, ranks and select answers above 2^31 and 2^32
bits, checked against the input itself (access, level-0 bits, occurrence
counts, first and last occurrence of every symbol)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_beyond_2p31_symbols(wtg):
    n, L = 3 * (1 << 30) + 37, 3
    rng = np.random.default_rng(31)
    sym = rng.integers(0, 1 << L, n, dtype=np.uint8)
    t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    # access, including the last positions
    idx = np.concatenate([rng.integers(0, n, 1 << 16), np.arange(n - 64, n)]).astype(np.uint64)
    assert np.array_equal(t.access(idx), sym[idx.astype(np.int64)].astype(np.uint64))
    # level 0 is the top bit of every symbol, in input order: check both ends
    bits = t.bits()
    for lo in (0, n - (1 << 20) - 5):
        w0, w1 = lo // 64, (lo + (1 << 20)) // 64 + 1
        got = np.unpackbits(bits[w0:w1].view(np.uint8), bitorder="little")[lo - 64 * w0:lo - 64 * w0 + (1 << 20)]
        assert np.array_equal(got, (sym[lo:lo + (1 << 20)] >> (L - 1)) & 1)
    # occurrences, first and last occurrence of every symbol
    counts = np.bincount(sym, minlength=1 << L)
    cs = np.arange(1 << L, dtype=np.uint64)
    assert np.array_equal(t.rank(np.full(1 << L, n, dtype=np.uint64), cs), counts.astype(np.uint64))
    first = t.select(np.ones(1 << L, dtype=np.uint64), cs)
    last = t.select(counts.astype(np.uint64), cs)
    tail = sym[n - (1 << 16):]
    for c in range(1 << L):
        assert int(first[c]) == int(np.argmax(sym[: 1 << 16] == c))
        assert int(last[c]) == n - (1 << 16) + int(np.flatnonzero(tail == c)[-1])
    # the select support counts every one of the concatenated bitvector
    assert t.select_tables(1).arg_cnt + t.select_tables(0).arg_cnt == n * L
