"""Generate tests/golden/golden64.npz from the FFTW-backed oracle.

The oracle restates the reference's 2D path in C; its FFTW-backed version routes every
transform through FFTW 3.3.9 compiled from the reference's own vendored sources
(oracle/_ref, made by ``make -C oracle ref``), planned FFTW_ESTIMATE per
transform as src/derive2csh.f95:73-106 does.  The fixtures pin the portable
own-FFT oracle (tests/test_oracle.py) and the GPU path (tests/test_gpu_*.py).

Run from the repository root:  python tests/golden/make_golden.py [2d] [3d] [coh] [com]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden64.npz"


def main() -> None:
    O = orc.load(fftw=True)
    assert O.is_fftw
    rng = np.random.default_rng(20240512)
    g: dict[str, np.ndarray] = {}
    n = 64
    # FFT vectors: rectangular real field, and a non-Hermitian half spectrum
    x = rng.standard_normal((32, 64))
    g["fft_r2c_in"] = x
    g["fft_r2c_out"] = O.r2c(x)
    c = rng.standard_normal((64, 17)) + 1j * rng.standard_normal((64, 17))
    g["fft_c2r_in"] = c
    g["fft_c2r_out"] = O.c2r(c)
    # configuration-1 initial condition (src/main2css.f95:78-110): 64^2, Lx=Ly=2 (x pi),
    # W0=25, m0=2, d=3/128 written as 0.0234375
    w_real = O.ic_shear(n, n, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=0)
    g["ic_real"] = w_real
    w0 = O.r2c(w_real)
    g["ic_spec"] = w0
    # one RHS evaluation of each kind
    g["rhs_plain"] = O.derive2csh(w0, 0.01)
    O.set_css_params(2 * orc.PI_R4, 2 * orc.PI_R4, 10.0)
    g["rhs_screen"] = O.derive2css(w0, 1.0, 0.01)
    O.set_css_params(2.0 * orc.PI_R8, 2.0 * orc.PI_R8, 10.0)
    g["rhs_screen_driverL"] = O.derive2css(w0, 1.0, 0.01)
    O.set_css_params(2 * orc.PI_R4, 2 * orc.PI_R4, 10.0)
    # AB2 runs with the driver's history rotation (zero history before step 1)
    for steps in (1, 10, 2000):
        w, fo = O.run(w0, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=steps)
        g[f"ab2_plain_{steps}"] = w
        g[f"ab2_plain_{steps}_hist"] = fo
    w, _ = O.run(w0, rhs=1, scheme=0, alpha=1.0, nu=0.01, dt=1e-4, steps=2000)
    g["ab2_screen_2000"] = w
    # RK4: plain RHS from a seeded random-phase spectrum, and one rk42css step
    wr = O.ic_random(n, n, 6.0, 0.5, 20240512)
    g["ic_random"] = wr
    w, _ = O.run(wr, rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=10)
    g["rk4_plain_10"] = w
    g["rk42css_1"] = O.rk42css(w0, 1.0, 0.01, 1e-4)
    # diagnostics
    g["energy_enstrophy_ic"] = np.array(O.energy_enstrophy(w0))
    g["diag_css_ic"] = O.diag_css(w0, 2.0 * orc.PI_R8, 2.0 * orc.PI_R8, 10.0)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")




def main3d() -> None:
    """tests/golden/golden3d.npz: the 3D MHD path at 16^3 from the FFTW oracle
    (reference initial condition of src/main3com.f95:292-347, faithful 1/450)."""
    O = orc.load(fftw=True)
    out = Path(__file__).resolve().parent / "golden3d.npz"
    real = O.ic3d_abc(16, 16, 16)
    state = O.state_from_real(real)
    p = orc.mhd_params()
    g = {"state0": state, "derive_faithful": O.derive3com(state, p)}
    st, h = O.run3d(state, p, 1e-3, 5)
    g["ab2_5"] = st
    np.savez_compressed(out, **g)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


def main_coh() -> None:
    """tests/golden/golden_coh.npz: the 2D compressible isothermal path at 64^2
    from the FFTW oracle: the driver's initial state (src/main2coh.f95:140-210),
    one derive2coh of it and of a seeded smooth state, and AB2 runs with the
    driver's parameters (mux = muy = 2e-4, CS = 3.77, 2 pi box, dt = 1e-3)."""
    O = orc.load(fftw=True)
    out = Path(__file__).resolve().parent / "golden_coh.npz"
    p = orc.coh_params()
    st = O.ic_coh(64, 64)
    g = {"ic": st, "rhs_ic": O.derive2coh(st, p)}
    rng = np.random.default_rng(20240601)
    n = 64
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    kx = np.arange(n // 2 + 1)[None, :]
    env = np.exp(-(kx**2 + ky**2) / 18.0)
    sm = np.stack([env * (rng.standard_normal((n, n // 2 + 1)) + 1j * rng.standard_normal((n, n // 2 + 1)))
                   for _ in range(3)]) * 40.0
    sm[0, 0, 0] = n * n  # mean density 1
    g["smooth"] = sm
    g["rhs_smooth"] = O.derive2coh(sm, orc.coh_params(mux=1e-3, muy=5e-4, cs=2.0))
    for steps in (1, 10, 2000):
        s2, h2 = O.run_coh(st, p, 1e-3, steps)
        g[f"ab2_{steps}"] = s2
        g[f"ab2_{steps}_hist"] = h2
    np.savez_compressed(out, **g)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


def smooth_com_state(O, n: int, seed: int) -> np.ndarray:
    """A smooth six-field MHD state: rho = 1 + 0.05 r, u and B fluctuations of
    order 0.3 about B0 = 1, E = P/(2/3) + kinetic + magnetic with CS = 100."""
    rng = np.random.default_rng(seed)
    x = np.arange(n) * (2 * np.pi / n)
    X, Y = np.meshgrid(x, x)  # [y][x]

    def field():
        f = np.zeros((n, n))
        for _ in range(6):
            kx, ky = rng.integers(-3, 4, size=2)
            f += rng.standard_normal() * np.cos(kx * X + ky * Y + rng.uniform(0, 2 * np.pi))
        return f / 6.0

    rho = 1.0 + 0.05 * field()
    ux, uy = 0.3 * field(), 0.3 * field()
    bx, by = 1.0 + 0.3 * field(), 1.0 + 0.3 * field()
    E = 100.0**2 * rho / (5.0 / 3.0 - 1.0) + 0.5 * rho * (ux * ux + uy * uy) + 0.5 * (bx * bx + by * by)
    return np.stack([O.r2c(f) for f in (rho, rho * ux, rho * uy, E, bx, by)])


def main_com() -> None:
    """tests/golden/golden_com.npz: the 2D compressible MHD path at 64^2 from the
    FFTW oracle: the driver's initial state (src/main2com.f95:229-291), one
    derive2com of it and of a smooth state in the faithful and the defined mode,
    and AB2 runs from the initial state (mu = 1e-3, eta = 1e-4, CS = 100,
    kf = A = 1, dt = 2e-4)."""
    O = orc.load(fftw=True)
    out = Path(__file__).resolve().parent / "golden_com.npz"
    st = O.ic_com(64, 64)
    g = {"ic": st, "rhs_ic": O.derive2com(st, orc.com_params())}
    sm = smooth_com_state(O, 64, 20240602)
    g["smooth"] = sm
    g["rhs_smooth"] = O.derive2com(sm, orc.com_params())
    g["rhs_smooth_defined"] = O.derive2com(sm, orc.com_params(defined=1))
    for steps in (1, 10, 500):
        s2, h2 = O.run_com(st, orc.com_params(), 2e-4, steps)
        g[f"ab2_{steps}"] = s2
        g[f"ab2_{steps}_hist"] = h2
    s2, _ = O.run_com(sm, orc.com_params(defined=1), 2e-4, 50)
    g["ab2_smooth_defined_50"] = s2
    np.savez_compressed(out, **g)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    import sys as _sys

    which = _sys.argv[1:] or ["2d", "3d", "coh", "com"]
    if "2d" in which:
        main()
    if "3d" in which:
        main3d()
    if "coh" in which:
        main_coh()
    if "com" in which:
        main_com()
