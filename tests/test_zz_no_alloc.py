"""GPU test of tara_derive2csh_noalloc, the allocation-free variant of the plain
RHS for callers that cannot call cudaMalloc (their device memory belongs to
another allocator or is reserved up front, or they must avoid the device-wide
synchronisation an allocation can cause).

The test owns the device buffers (torch allocates them; the entry point itself
allocates nothing) and compares the variant's output with the existing
derive2csh_ drop-in, within the 1e-12 tolerance of the other RHS tests, on two
calls in a row.  Its file name sorts last so that a run stopping at the first
failure has already run every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _noalloc(w: np.ndarray, nu: float) -> np.ndarray:
    import torch

    ny, nh = w.shape
    nx = 2 * (nh - 1)
    dev_in = torch.from_numpy(np.ascontiguousarray(w).view(np.float64).copy()).cuda()
    dev_out = torch.full_like(dev_in, float("nan"))  # anything unwritten stays NaN
    stream = torch.cuda.current_stream()
    rc = tg.lib().tara_derive2csh_noalloc(nx, ny, nu, ctypes.c_void_p(dev_in.data_ptr()),
                                          ctypes.c_void_p(dev_out.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream))
    assert rc == tg.TARA_OK, tg.last_error()
    stream.synchronize()
    return dev_out.cpu().numpy().view(np.complex128).reshape(ny, nh)


def test_noalloc_matches_dropin_two_calls(golden):
    # two calls in a row on different inputs: the second must not see the first
    cases = [(golden["ic_spec"], 0.01), (golden["ab2_plain_10"], 0.02)]
    for w, nu in cases:
        ref = tg.derive2csh(w, nu)
        out = _noalloc(w, nu)
        assert np.all(np.isfinite(out))
        assert rel_l2(out, ref) < 1e-12


def test_noalloc_sizes_share_the_scratch():
    # the largest supported grid, then a smaller rectangular one, then the largest again
    rng = np.random.default_rng(17)
    for ny, nx in ((256, 256), (32, 64), (256, 256)):
        w = np.fft.rfft2(rng.standard_normal((ny, nx)))
        assert rel_l2(_noalloc(w, 1e-3), tg.derive2csh(w, 1e-3)) < 1e-12


def test_noalloc_rejects_oversize_grid():
    rc = tg.lib().tara_derive2csh_noalloc(512, 512, 0.01, None, None, None)
    assert rc == tg.TARA_ERR_ARGS
    assert "256" in tg.last_error()[1]
