"""Failure handling, made on the host only (no GPU fault, trap or hang).

* A bounded look-back wait that runs out: the rank/select pass over a caller
  bitvector is started with its tile counter at 1, so tile 0 never publishes
  its count (a flag that nothing sets); with the wait limit lowered, every
  other tile gives up, the kernel returns, the build reports ERR_TIMEOUT, and
  the next build on the same context is bit-exact again.
* Device allocation failures injected at every allocation of a build: the
  build returns ERR_OOM and frees what it holds, a handle being rebuilt can
  still be freed, and later builds are unaffected.
The reference has no device waits; its error sites throw std::logic_error
(wt_int/wt_int_par.hpp:377,645), which the C++ layer maps from these codes.
"""
import time

import numpy as np
import pytest

import datagen


def test_hooks_are_host_side(wtg):
    # arming and disarming needs no GPU; a negative countdown is refused
    wtg.inject_alloc_failure(0)
    wtg.inject_lookback_stall(False)
    with pytest.raises(wtg.WtgError) as e:
        wtg.inject_alloc_failure(-1)
    assert e.value.code == wtg.ERR_INVALID


@pytest.mark.gpu
def test_lookback_wait_runs_out_and_context_survives(wtg, oracle):
    size = (1 << 22) + 123  # 33 tiles of the rank/select pass
    words = datagen.random_bits(size, 0.3, seed=5)
    wtg.set_wait_limits(lookback_spins=2000)
    try:
        wtg.inject_lookback_stall(True)
        t0 = time.perf_counter()
        with pytest.raises(wtg.WtgError) as e:
            wtg.BitVectorSupport(words, size, wtg.RANK)
        assert e.value.code == wtg.ERR_TIMEOUT
        assert time.perf_counter() - t0 < 30
    finally:
        wtg.inject_lookback_stall(False)
        wtg.set_wait_limits(0, 0)
    # the context is still usable and the same build is exact
    w = np.concatenate([words, np.zeros(1, np.uint64)])
    b = wtg.BitVectorSupport(words, size, wtg.ALL)
    assert np.array_equal(b.rank_table(), oracle.rank_build(w, size))
    s = oracle.Select(w, size, 1)
    assert np.array_equal(b.select_tables(1).pool, s.pool)
    b.free()


@pytest.mark.gpu
def test_injected_allocation_failures(wtg, oracle):
    sym = datagen.exp_u32(70001, seed=9)
    L = 20
    bits, _ = oracle.wt_build(sym, L)
    failures = 0
    try:
        for k in range(1, 200):
            wtg.inject_alloc_failure(k)
            try:
                t = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
            except wtg.WtgError as e:
                assert e.code == wtg.ERR_OOM
                failures += 1
                continue
            # k is past the build's last allocation: the build is whole
            assert np.array_equal(t.bits(), bits)
            t.free()
            break
        else:
            pytest.fail("a build made more than 200 device allocations")
    finally:
        wtg.inject_alloc_failure(0)
    assert failures >= 5
    # a handle that fails while being rebuilt can still be freed
    import torch
    d = torch.from_numpy(sym.view(np.int32).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    t = wtg.WaveletTree.from_device(d.data_ptr(), sym.size, 4, L, wtg.ALL, stream)
    t.sync()
    big = torch.from_numpy(datagen.exp_u32(1 << 20, seed=10).view(np.int32).copy()).cuda()
    wtg.inject_alloc_failure(1)
    try:
        with pytest.raises(wtg.WtgError) as e:
            wtg.WaveletTree.from_device(big.data_ptr(), 1 << 20, 4, L, wtg.ALL, stream, tree=t)
        assert e.value.code == wtg.ERR_OOM
    finally:
        wtg.inject_alloc_failure(0)
    t.free()
    t2 = wtg.WaveletTree(sym, levels=L, flags=wtg.ALL)
    assert np.array_equal(t2.bits(), bits)
    t2.free()
