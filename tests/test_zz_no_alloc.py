"""The allocation-free skinny product (qflex_gb300_multiply_skinny_noalloc)
against the regular entry point (qflex_gb300_multiply) through the C ABI.

This file is named to be collected last, so that a run stopping at the
first failure has already run every other test. It passes on its own in a
fresh process too: the entry point needs no context and sets itself up on
its first call. With lazy module loading that first call may also load the
library's device code (which places the fixed array), so the free-memory
comparison starts after one warm-up call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# Dot products, matrix-vector products with long rows / columns, and the
# largest output count the entry point accepts.
SHAPES = [(1, 1, 100000), (4, 1, 30000), (1, 8, 20000), (8, 8, 65536), (64, 1, 1 << 20), (2, 3, 5)]


def _data(torch, m, n, k, seed):
    g = np.random.default_rng(seed)
    A = (g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))).astype(np.complex64)
    B = (g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))).astype(np.complex64)
    return torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_noalloc_matches_regular_entry_point_twice(built_lib, m, n, k):
    import torch
    from qflex_gb300 import Context
    from qflex_gb300._lib import multiply_skinny_noalloc
    assert torch.cuda.is_available()
    ctx = Context(0)
    # Warm-up: the first call on a device may load the module and place the
    # fixed array; later calls must not change the device's free memory.
    wA, wB = _data(torch, m, n, k, seed=7)
    warm = torch.empty((m, n), dtype=torch.complex64, device="cuda")
    multiply_skinny_noalloc(wA.data_ptr(), wB.data_ptr(), warm.data_ptr(), m, n, k, 0)
    torch.cuda.synchronize()
    for call in range(2):  # two calls in a row, different data
        dA, dB = _data(torch, m, n, k, seed=1000 * call + m + n + k)
        want = torch.zeros((m, n), dtype=torch.complex64, device="cuda")
        got = torch.full((m, n), float("nan"), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        ctx.multiply(dA.data_ptr(), dB.data_ptr(), want.data_ptr(), m, n, k)
        ctx.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        cached_before = torch.cuda.memory_reserved()
        multiply_skinny_noalloc(dA.data_ptr(), dB.data_ptr(), got.data_ptr(), m, n, k, 0)
        torch.cuda.synchronize()
        # Nothing was allocated: neither through the driver (the device's
        # free memory, which only this process uses on a GPU of its own) nor
        # through torch's caching allocator.
        assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.cuda.memory_reserved() == cached_before
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.isfinite(g).all()
        # Same FP32 partial sums, possibly split differently: FP32 rounding
        # of a k-term sum of unit-variance products.
        assert np.max(np.abs(g - w)) <= 2e-6 * np.sqrt(k) + 1e-6, (m, n, k, call)


def test_noalloc_rejects_too_many_outputs(built_lib):
    import torch
    from qflex_gb300 import QflexGb300Error
    from qflex_gb300._lib import multiply_skinny_noalloc
    dA, dB = _data(torch, 16, 16, 8, 0)
    out = torch.zeros((16, 16), dtype=torch.complex64, device="cuda")
    with pytest.raises(QflexGb300Error) as e:
        multiply_skinny_noalloc(dA.data_ptr(), dB.data_ptr(), out.data_ptr(), 16, 16, 8)
    assert "at most 64 outputs" in str(e.value)
    # m * n would wrap to 0 in 64 bits: still rejected, nothing launched.
    with pytest.raises(QflexGb300Error) as e:
        multiply_skinny_noalloc(dA.data_ptr(), dB.data_ptr(), out.data_ptr(), 1 << 32, 1 << 32, 8)
    assert "at most 64 outputs" in str(e.value)
