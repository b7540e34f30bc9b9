"""GPU tests of the input.ini driver (tara_run_ini): the screened and plain 2D
loops, the 2D compressible hydro and MHD loops and the 3D MHD loop, their output files checked against the oracle run on
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


INI2C = """[dimension]
dim = 2
[architecture]
arch = cpu
[parallel]
mode = openmp
[type]
domain = {domain}
[problem]
hydrotype = bare
[grid]
Nx = 64
Ny = 64
[length]
Lx = 2.0d0
Ly = 2.0d0
[resistivity]
nu = {nu}
[time]
time_min = 0.0d0
time_max = 1.0d0
dt = {dt}
"""


def _grid_fields(O, spectra):
    nn = 64.0 * 64.0
    return [O.c2r(a) / nn for a in spectra]


def _ik(n):
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    kx = np.arange(n // 2 + 1)[None, :].astype(float)
    return kx, ky


def test_coh_driver_matches_oracle(tmp_path, oracle):
    """tara2dHydOMP (src/main2coh.f95): Energy.dat every step, the snapshot at t = 0."""
    steps = 12
    out = run(tmp_path, INI2C.format(domain="hydro", nu="0.010d0", dt="0.0010d0"), steps)
    e = rows(out / "Energy.dat")
    assert e.shape == (steps, 7)
    assert np.allclose(e[:, 0], np.arange(steps) * 1e-3, rtol=0, atol=1e-15)
    p = orc.coh_params()  # the driver's mux = muy = 0.0002 whatever the ini's nu
    st = oracle.ic_coh(64, 64)
    kx, ky = _ik(64)
    h = None
    for s in range(steps):
        st, h = oracle.run_coh(st, p, 1e-3, 1, hist=h)
        om_k = 1j * kx * st[2] - 1j * ky * st[1]
        n, ux, uy, om = _grid_fields(oracle, [st[0], st[1], st[2], om_k])
        nn = 64.0 * 64.0
        ref = [np.sum(ux * ux + uy * uy) / (2 * nn), np.sum(uy * uy) / (2 * nn), 1.0, np.sum(om) / nn,
               np.sum(om**2) / nn, np.sum(om**3) / nn]
        scale = [ref[0], ref[1], 1.0, np.sum(np.abs(om)) / nn, ref[4], np.sum(np.abs(om) ** 3) / nn]
        for c in range(1, 7):
            assert abs(e[s, c] - ref[c - 1]) <= 1e-10 * scale[c - 1], (s, c)
        if s == 0:
            snap0 = np.stack([om.T.ravel(), n.T.ravel(), ux.T.ravel(), uy.T.ravel()], axis=1)
    snap = rows(out / "fort.00000100")  # t = 0, written after the first step
    assert snap.shape == (64 * 64, 6)
    assert np.abs(snap[:, 2:] - snap0).max() < 1e-10 * np.abs(snap0).max()
    init = rows(out / "Initial_Grid_Data_Reproduced.dat")
    assert init.shape == (64 * 64, 6)
    st0 = oracle.ic_coh(64, 64)
    n0, ux0, uy0 = _grid_fields(oracle, [st0[0], st0[1], st0[2]])
    assert np.abs(init[:, 3] - n0.T.ravel()).max() < 1e-12
    assert np.abs(init[:, 4] - ux0.T.ravel()).max() < 1e-10 * np.abs(ux0).max()


def test_com_driver_matches_oracle(tmp_path, oracle):
    """tara2dMHDOMP (src/main2com.f95): Energy.dat every 100 steps, fort.(t+100000) at t = 0."""
    steps = 201
    out = run(tmp_path, INI2C.format(domain="mhd", nu="0.0010d0", dt="0.00020d0"), steps)
    e = rows(out / "Energy.dat")
    assert e.shape == (3, 6)
    assert np.allclose(e[:, 0], [0.0, 100 * 2e-4, 200 * 2e-4], rtol=0, atol=1e-15)
    p = orc.com_params(mu=1e-3)
    st = oracle.ic_com(64, 64)
    kx, ky = _ik(64)
    nn = 64.0 * 64.0
    h = None
    row = 0
    for s in range(steps):
        st, h = oracle.run_com(st, p, 2e-4, 1, hist=h)
        if s % 100:
            continue
        rho, rux, ruy, E, bx, by = _grid_fields(oracle, list(st))
        ux, uy = rux / rho, ruy / rho
        uxk, uyk = oracle.r2c(ux), oracle.r2c(uy)
        om, jb, divb = _grid_fields(oracle, [1j * kx * uyk - 1j * ky * uxk, 1j * kx * st[5] - 1j * ky * st[4],
                                             1j * kx * st[4] + 1j * ky * st[5]])
        ref = [np.sum(ux * ux + uy * uy) / nn, np.sum(bx * bx + by * by) / nn, np.sum(om**2) / nn,
               np.sum(jb**2) / nn]
        for c in range(4):
            assert abs(e[row, c + 1] - ref[c]) <= 1e-9 * abs(ref[c]) + 1e-13, (s, c)
        assert abs(e[row, 5]) < 1e-12 and abs(np.sum(divb) / nn) < 1e-12
        if s == 0:
            snap0 = np.stack([f.T.ravel() for f in (rho, ux, uy, 100.0**2 * rho, E, bx, by)], axis=1)
        row += 1
    snap = rows(out / "fort.00100000")
    assert snap.shape == (64 * 64, 9)
    assert np.abs(snap[:, 2:] - snap0).max() < 1e-9 * np.abs(snap0).max()
