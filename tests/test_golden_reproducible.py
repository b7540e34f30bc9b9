"""The committed fixtures are what tests/golden/make_golden.py makes: where the
FFTW-backed oracle exists (oracle/_ref, built from the reference's vendored
FFTW sources; not on machines without the reference tree), its outputs for the
fixtures' inputs equal the stored arrays bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle as orc

pytestmark = pytest.mark.skipif(not orc.available(fftw=True), reason="FFTW-backed oracle not built here")
GOLD = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def ref():
    O = orc.load(fftw=True)
    assert O.is_fftw
    return O


def test_golden64_reproduces(ref):
    g = dict(np.load(GOLD / "golden64.npz"))
    assert np.array_equal(ref.r2c(g["fft_r2c_in"]), g["fft_r2c_out"])
    assert np.array_equal(ref.c2r(g["fft_c2r_in"]), g["fft_c2r_out"])
    w_real = ref.ic_shear(64, 64, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=0)
    assert np.array_equal(w_real, g["ic_real"])
    w0 = ref.r2c(w_real)
    assert np.array_equal(w0, g["ic_spec"])
    assert np.array_equal(ref.derive2csh(w0, 0.01), g["rhs_plain"])
    ref.set_css_params(2 * orc.PI_R4, 2 * orc.PI_R4, 10.0)
    assert np.array_equal(ref.derive2css(w0, 1.0, 0.01), g["rhs_screen"])
    w, fo = ref.run(w0, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=10)
    assert np.array_equal(w, g["ab2_plain_10"]) and np.array_equal(fo, g["ab2_plain_10_hist"])
    wr = ref.ic_random(64, 64, 6.0, 0.5, 20240512)
    assert np.array_equal(wr, g["ic_random"])
    w, _ = ref.run(wr, rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=10)
    assert np.array_equal(w, g["rk4_plain_10"])


def test_golden_coh_reproduces(ref):
    g = dict(np.load(GOLD / "golden_coh.npz"))
    st = ref.ic_coh(64, 64)
    assert np.array_equal(st, g["ic"])
    assert np.array_equal(ref.derive2coh(st, orc.coh_params()), g["rhs_ic"])
    s2, h2 = ref.run_coh(st, orc.coh_params(), 1e-3, 10)
    assert np.array_equal(s2, g["ab2_10"]) and np.array_equal(h2, g["ab2_10_hist"])


def test_golden_com_reproduces(ref):
    g = dict(np.load(GOLD / "golden_com.npz"))
    st = ref.ic_com(64, 64)
    assert np.array_equal(st, g["ic"])
    assert np.array_equal(ref.derive2com(st, orc.com_params()), g["rhs_ic"])
