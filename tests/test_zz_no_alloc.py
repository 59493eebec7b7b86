"""wtg_rank_build_noalloc: the rank table built without device allocation
(for callers that cannot allocate: its scratch is a fixed array inside the
library) matches the table of the allocating path, on two calls in a row,
through the C ABI.  Kept in a file collected last."""
import numpy as np
import pytest

import datagen

pytestmark = pytest.mark.gpu


def _device_words(torch, words):
    w = np.concatenate([words, np.zeros(1, np.uint64)])
    return torch.from_numpy(w.view(np.int64).copy()).cuda()


@pytest.mark.parametrize("size,dens", [(1000, 0.5), (262144, 0.3), ((1 << 22) + 77, 0.01)])
def test_noalloc_rank_matches_allocating_build(wtg, size, dens):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    for call, seed in enumerate((size, size + 1)):  # two calls in a row, different inputs
        words = datagen.random_bits(size, dens, seed=seed)
        expected = wtg.BitVectorSupport(words, size, wtg.RANK).rank_table()
        d_words = _device_words(torch, words)
        d_rank = torch.full((wtg.rank_words(size),), -1, dtype=torch.int64, device="cuda")
        wtg.rank_build_noalloc(d_words.data_ptr(), size, d_rank.data_ptr(), stream)
        got = d_rank.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, expected), f"call {call}"


def test_noalloc_rejects_oversized_input(wtg):
    torch = pytest.importorskip("torch")
    d = torch.zeros(4, dtype=torch.int64, device="cuda")
    with pytest.raises(wtg.WtgError) as e:
        wtg.rank_build_noalloc(d.data_ptr(), (1 << 34) + 1, d.data_ptr())
    assert e.value.code == wtg.ERR_RANGE
