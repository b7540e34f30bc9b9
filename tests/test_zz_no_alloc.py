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
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _enqueue(w: np.ndarray, nu: float, stream):
    """Copy w to the device and enqueue one call on `stream` (no host wait);
    returns the output tensor and the input tensor (kept alive until the sync)."""
    import torch

    ny, nh = w.shape
    nx = 2 * (nh - 1)
    with torch.cuda.stream(stream):
        dev_in = torch.from_numpy(np.ascontiguousarray(w).view(np.float64).copy()).cuda()
        dev_out = torch.full_like(dev_in, float("nan"))  # anything unwritten stays NaN
    rc = tg.lib().tara_derive2csh_noalloc(nx, ny, nu, ctypes.c_void_p(dev_in.data_ptr()),
                                          ctypes.c_void_p(dev_out.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream))
    assert rc == tg.TARA_OK, tg.last_error()
    return dev_out, dev_in


def _to_spec(dev_out, ny: int, nh: int) -> np.ndarray:
    return dev_out.cpu().numpy().view(np.complex128).reshape(ny, nh)


def _noalloc(w: np.ndarray, nu: float) -> np.ndarray:
    import torch

    stream = torch.cuda.current_stream()
    out, _ = _enqueue(w, nu, stream)
    stream.synchronize()
    return _to_spec(out, *w.shape)


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


def test_noalloc_back_to_back_on_one_stream():
    """Calls one after another on one stream are the documented safe use: the
    second call rewrites the shared tables only after the first call's kernels
    (stream order), so both outputs are right with a single sync at the end."""
    import torch

    rng = np.random.default_rng(23)
    w1 = np.fft.rfft2(rng.standard_normal((256, 256)))
    w2 = np.fft.rfft2(rng.standard_normal((64, 128)))
    stream = torch.cuda.Stream()
    out1, keep1 = _enqueue(w1, 1e-3, stream)
    out2, keep2 = _enqueue(w2, 2e-3, stream)
    stream.synchronize()
    assert rel_l2(_to_spec(out1, *w1.shape), tg.derive2csh(w1, 1e-3)) < 1e-12
    assert rel_l2(_to_spec(out2, *w2.shape), tg.derive2csh(w2, 2e-3)) < 1e-12


def test_noalloc_nonfinite_is_not_reported():
    """A NaN in the input gives a non-finite right-hand side; as documented, the
    call still returns TARA_OK and the caller finds the NaN in its output."""
    rng = np.random.default_rng(29)
    w = np.fft.rfft2(rng.standard_normal((64, 64)))
    w[3, 5] = np.nan
    out = _noalloc(w, 1e-3)
    assert not np.all(np.isfinite(out))


_FRESH = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    import tara_gb300 as tg
    rng = np.random.default_rng(31)
    w = np.fft.rfft2(rng.standard_normal((128, 128)))
    stream = torch.cuda.Stream()  # non-blocking with respect to the legacy stream
    with torch.cuda.stream(stream):
        dev_in = torch.from_numpy(w.view(np.float64).copy()).cuda()
        dev_out = torch.full_like(dev_in, float("nan"))
    # the first call of this process: set-up (address, twiddle upload) happens here
    rc = tg.lib().tara_derive2csh_noalloc(128, 128, 1e-3, ctypes.c_void_p(dev_in.data_ptr()),
                                          ctypes.c_void_p(dev_out.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream))
    assert rc == tg.TARA_OK, tg.last_error()
    stream.synchronize()
    out = dev_out.cpu().numpy().view(np.complex128).reshape(w.shape)
    ref = tg.derive2csh(w, 1e-3)
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 1e-12, err
    print("ok", err)
""")


def test_noalloc_first_call_on_side_stream_in_fresh_process():
    """The first call of a process, on a non-blocking stream: the twiddle tables
    its set-up uploads must be in device memory before that stream's kernels
    read them."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok" in r.stdout
