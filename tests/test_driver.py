"""GPU tests of the input.ini driver (tara_run_ini): the screened and plain 2D
loops and the 3D MHD loop, their output files checked against the oracle run on
the same inputs (relative tolerance 1e-10 after the stated number of steps)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import tara_gb300 as tg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
PI = orc.PI_R8

INI2D = """[dimension]
dim = 2
[architecture]
arch = cpu
[parallel]
mode = serial
[type]
domain = hydro
[problem]
hydrotype = {hydro}
[particle]
Np = 10
[grid]
Nx = 64
Ny = 64
Nz = 64
[length]
Lx = 2.0d0
Ly = 2.0d0
Lz = 2.0d0
[resistivity]
nu = 0.010d0
eta = 0.0d0
[time]
time_min = 0.0d0
time_max = 2.0d0
dt = 0.00010d0
[initialProfile]
W0 = 25.0d0
m0 = 2.0d0
d = 0.0234375d0
"""


def run(tmp_path, text, steps):
    ini = tmp_path / "input.ini"
    ini.write_text(text)
    out = tmp_path / "output"
    rc = tg.lib().tara_run_ini(str(ini).encode(), str(out).encode(), steps)
    assert rc == tg.TARA_OK, tg.last_error()
    return out


def rows(path: Path) -> np.ndarray:
    return np.array([[float(v) for v in line.split()] for line in path.read_text().splitlines()])


def fields(O, w, lam, screened):
    """psi, omega (k^2 psi when screened), ux, uy as the reference drivers form
    them (true pi, box 2 pi, lambda on the ky >= 0 half only when screened)."""
    n = w.shape[0]
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    kx = np.arange(n // 2 + 1)[None, :].astype(float)
    k2 = kx**2 + ky**2
    den = np.where(screened & (np.arange(n)[:, None] < n // 2), k2 + lam, k2)
    den[0, 0] = 1.0
    psi = w / den
    psi[0, 0] = 0
    om = k2 * psi if screened else w
    ux, uy = 1j * ky * psi, -1j * kx * psi
    nn = float(n * n)
    return [O.c2r(a) / nn for a in (psi, om, ux, uy)]


def test_screened_driver_matches_oracle(tmp_path, oracle):
    steps = 20
    out = run(tmp_path, INI2D.format(hydro="screen"), steps)
    e = rows(out / "Energy.dat")
    assert e.shape == (steps, 3)
    assert np.allclose(e[:, 0], np.arange(steps) * 1e-4, rtol=0, atol=1e-15)
    # oracle: IC of src/main2css.f95, derive2css in defined mode with the driver's box
    w = oracle.r2c(oracle.ic_shear(64, 64, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=0))
    oracle.set_css_params(2.0 * PI, 2.0 * PI, 10.0)
    fo = None
    ye = 0.0
    for s in range(steps):
        w, fo = oracle.run(w, rhs=1, scheme=0, alpha=1.0, nu=0.01, dt=1e-4, steps=1, dt_old=fo)
        d = oracle.diag_css(w, 2.0 * PI, 2.0 * PI, 10.0)
        ye += d[1]
        if s == 0:
            _, om, ux, uy = fields(oracle, w, 10.0, True)
    oracle.set_css_params(2 * orc.PI_R4, 2 * orc.PI_R4, 10.0)
    assert abs(e[-1, 1] - d[0]) < 1e-10 * d[0]
    assert abs(e[-1, 2] - ye) < 1e-10 * ye
    snap = rows(out / "fort.00000100")  # t = 0 -> unit 100, after the first step
    assert snap.shape == (64 * 64, 5)
    ref = np.stack([ux.T.ravel(), uy.T.ravel(), om.T.ravel()], axis=1)  # i outer, j inner
    assert np.abs(snap[:, 2:] - ref).max() < 1e-10 * np.abs(ref).max()
    init = rows(out / "Initial_Condition_Omega_REP.dat")
    assert init.shape == (64 * 64, 6)


def test_plain_driver_matches_oracle(tmp_path, oracle):
    out = run(tmp_path, INI2D.format(hydro="bare"), 3)
    assert (out / "Energy.dat").exists() and (out / "Energy.dat").read_text() == ""
    w0 = oracle.r2c(oracle.ic_shear(64, 64, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=1))
    w, _ = oracle.run(w0, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=1)
    _, om, ux, uy = fields(oracle, w, 0.0, False)
    snap = rows(out / "fort.00000100")
    ref = np.stack([om.T.ravel(), ux.T.ravel(), uy.T.ravel()], axis=1)
    assert np.abs(snap[:, 2:] - ref).max() < 1e-10 * np.abs(ref).max()
    x = np.arange(64) * (2 * PI / 64)
    assert np.allclose(snap[::64, 0], x, atol=1e-14)
    # Lagrangian particles (Np = 10): positions after the first step in fort.(0+105)
    r, _ = tg.park_miller(20)
    xp, yp = r[0::2].astype(np.float64) * (2 * PI), r[1::2].astype(np.float64) * (2 * PI)
    vx, vy = oracle.driver_velocity(w, 2 * PI, 2 * PI)
    xp, yp = oracle.particles_step(vx, vy, xp, yp, 2 * PI, 2 * PI, 1e-4)
    parts = rows(out / "fort.00000105")
    assert parts.shape == (10, 2)
    assert np.abs(parts - np.stack([xp, yp], axis=1)).max() < 1e-12


INI3D = """[dimension]
dim = 3
[architecture]
arch = cpu
[parallel]
mode = openmp
[type]
domain = mhd
[problem]
hydrotype = bare
[grid]
Nx = 16
Ny = 16
Nz = 16
[length]
Lx = 2.0d0
Ly = 2.0d0
Lz = 2.0d0
[resistivity]
nu = 0.010d0
[time]
time_min = 0.0d0
time_max = 1.0d0
dt = 0.0010d0
"""


def test_mhd3d_driver_matches_oracle(tmp_path, oracle):
    steps = 3
    out = run(tmp_path, INI3D, steps)
    e = rows(out / "Energy.dat")
    assert e.shape == (steps, 5)
    st = oracle.state_from_real(oracle.ic3d_abc(16, 16, 16))
    st, _ = oracle.run3d(st, orc.mhd_params(mu=0.01), 1e-3, steps)
    real = np.stack([oracle.c2r3(f) / 16**3 for f in st])
    rho, rux, ruy, ruz, E, bx, by, bz = real
    u2 = (rux / rho) ** 2 + (ruy / rho) ** 2 + (ruz / rho) ** 2
    ref = [100.0 * rho.mean(), 0.5 * u2.mean(), E.mean(), 0.5 * (bx**2 + by**2 + bz**2).mean()]
    assert np.allclose(e[-1, 1:], ref, rtol=1e-10)
