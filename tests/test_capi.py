"""The C-ABI library loads and exports every entry point include/wtg.h
declares; without a GPU the product path fails loudly (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared():
    src = open(os.path.join(ROOT, "include", "wtg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|uint64_t|const char\*)\s+(wtg_\w+)\(", src, re.M)))


def test_exports_every_declared_symbol(wtg):
    names = declared()
    assert len(names) >= 30
    lib = ctypes.CDLL(wtg.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing
    assert set(names) == set(wtg._SIGS)


def test_version_and_errors(wtg):
    assert wtg.lib().wtg_version() >= 100
    with pytest.raises(ValueError):
        wtg.WaveletTree(np.zeros(10, dtype=np.int32))
    with pytest.raises(wtg.WtgError) as e:
        wtg.WaveletTree(np.zeros(10, dtype=np.uint8), levels=25)
    assert e.value.code == wtg.ERR_INVALID


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour on a machine without a GPU")
def test_no_gpu_fails_loudly(wtg):
    with pytest.raises(wtg.WtgError) as e:
        wtg.WaveletTree(np.arange(100, dtype=np.uint8), levels=7)
    assert e.value.code == wtg.ERR_CUDA
    with pytest.raises(wtg.WtgError):
        wtg.BitVectorSupport(np.zeros(4, dtype=np.uint64), 200)


def test_levels_for_sigma(wtg, oracle):
    for s in [1, 2, 3, 4, 5, 7, 8, 9, 255, 256, 257, 1 << 20, (1 << 20) + 1]:
        assert wtg.levels_for_sigma(s) == oracle.levels_for_sigma(s)
