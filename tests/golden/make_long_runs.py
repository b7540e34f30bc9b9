"""Generate the long-run fixtures, computed by the FFTW-backed oracle:

tests/golden/long_rk4.npz   the 1000-step RK4 runs of the plain 2D solver at
                            512^2 and 2048^2;
tests/golden/long_mhd3d.npz the 500-step AB2 runs of the 3D compressible MHD
                            solver at 64^3 and 128^3 from the Orszag-Tang-type
                            initial state (oracle_ic3d_ot: amp 0.01, |k| <= 4,
                            seed 3), defined mode nu = eta = 0.01, dt = 1e-3
                            (src/derive3com.f95:6-1047, src/ab3com.f95:31-62
                            with the viscosity and resistivity from the
                            configuration instead of the hard-coded 1/450);
tests/golden/long_ensemble.npz  2000 RK4 steps of six runs of the 384-run
                            ensemble (runs 0, 1 at 128^2; 128, 129 at 256^2;
                            256, 257 at 512^2): nu = 1e-3, dt = 1e-4, E = 0.5,
                            seed 4000 + r, k0 = U[4, 10] from numpy
                            default_rng(4000) (the r-th of 384 draws).

Workload: box 2 pi x 2 pi, nu = 1e-4, dt = 5e-5, classic RK4 over the plain
right-hand side (src/derive2csh.f95:19-145; the rk42css signature,
src/rk42css.f95:6-52, integrates nothing in the reference, so the oracle's
classic RK4 is the definition), seeded random-phase initial vorticity with
E(k) ~ k^4 exp(-(k/6)^2) and total energy 0.5, seeds 20240512 (512^2) and
20242048 (2048^2).  Every transform goes through FFTW 3.3.9 compiled from the
reference's vendored sources (oracle/_ref), planned FFTW_ESTIMATE per
transform like the reference.

A full 2048^2 state is 33.6 MB, so the fixture keeps what a parity test needs
and nothing more: the energy and enstrophy after 0, 100 and 1000 steps, and the
real-space vorticity omega(x, y) on a 128 x 128 sub-lattice (every 16th point
at 2048^2, every 4th at 512^2) after 100 and 1000 steps.  The sub-lattice of
omega is a linear function of the full state, so a state that differs from the
oracle's by a relative L2 error e in the spectrum differs here by about e too.

Run from the repository root (about an hour on 8 cores, FFTW single-threaded as
the reference runs it; the pointwise loops use OpenMP):

    python tests/golden/make_long_runs.py [512] [2048] [mhd64] [mhd128] [ens]

Each 3D checkpoint keeps the eight fields (rho, rho u, E, B) on the grid at a
16^3 sub-lattice (every n/16-th point along each axis), so that each field is
compared on its own.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent / "long_rk4.npz"
OUT3 = Path(__file__).resolve().parent / "long_mhd3d.npz"
MHD_DT, MHD_CHECKPOINTS = 1e-3, (100, 500)
OUTE = Path(__file__).resolve().parent / "long_ensemble.npz"
ENS_RUNS, ENS_STEPS, ENS_NU, ENS_DT = (0, 1, 128, 129, 256, 257), 2000, 1e-3, 1e-4


def ensemble_run(r: int) -> tuple[int, float, int]:
    """(n, k0, seed) of run r of the 384-run ensemble (128 each at 128^2, 256^2, 512^2)."""
    k0 = np.random.default_rng(4000).uniform(4.0, 10.0, 384)
    return (128, 256, 512)[r // 128], float(k0[r]), 4000 + r
NU, DT, K0, ENERGY = 1e-4, 5e-5, 6.0, 0.5
SEEDS = {512: 20240512, 2048: 20242048}
CHECKPOINTS = (100, 1000)


def sub_lattice(O, w, n):
    stride = n // 128
    return O.c2r(w)[::stride, ::stride] / float(n * n)


def run_size(O, n: int, g: dict) -> None:
    w = O.ic_random(n, n, K0, ENERGY, SEEDS[n])
    e, z = O.energy_enstrophy(w)
    g[f"n{n}_energy_0"], g[f"n{n}_enstrophy_0"] = np.float64(e), np.float64(z)
    hist = None
    done = 0
    for step in CHECKPOINTS:
        t = time.time()
        w, hist = O.run(w, rhs=0, scheme=1, nu=NU, dt=DT, steps=step - done, dt_old=hist)
        done = step
        e, z = O.energy_enstrophy(w)
        g[f"n{n}_energy_{step}"], g[f"n{n}_enstrophy_{step}"] = np.float64(e), np.float64(z)
        g[f"n{n}_omega_{step}"] = sub_lattice(O, w, n)
        print(f"{n}^2: {step} steps, E={e:.15e} Z={z:.15e} ({time.time() - t:.0f} s)", flush=True)


def mhd_sub_lattice(O, st, n):
    s = n // 16
    return np.stack([O.c2r3(f)[::s, ::s, ::s] / float(n**3) for f in st])


def run_mhd(O, n: int, g: dict) -> None:
    p = orc.mhd_params(defined=1, nu_u=0.01, eta_b=0.01)
    st = O.ic3d_ot(n, amp=0.01, kmax=4, seed=3)
    g[f"mhd{n}_fields_0"] = mhd_sub_lattice(O, st, n)
    hist, done = None, 0
    for step in MHD_CHECKPOINTS:
        t = time.time()
        st, hist = O.run3d(st, p, MHD_DT, step - done, hist)
        done = step
        g[f"mhd{n}_fields_{step}"] = mhd_sub_lattice(O, st, n)
        print(f"mhd {n}^3: {step} steps ({time.time() - t:.0f} s)", flush=True)


def run_ensemble(O, g: dict) -> None:
    for r in ENS_RUNS:
        t = time.time()
        n, k0, seed = ensemble_run(r)
        w = O.ic_random(n, n, k0, ENERGY, seed)
        w, _ = O.run(w, rhs=0, scheme=1, nu=ENS_NU, dt=ENS_DT, steps=ENS_STEPS)
        g[f"run{r}_omega"] = sub_lattice(O, w, n)
        print(f"ensemble run {r} ({n}^2, k0={k0:.4f}): {ENS_STEPS} steps ({time.time() - t:.0f} s)",
              flush=True)


def main() -> None:
    args = sys.argv[1:] or ["512", "2048", "mhd64", "mhd128", "ens"]
    O = orc.load(fftw=True)
    assert O.is_fftw
    O.set_threads(8)
    for a in args:
        if a == "ens":
            out = OUTE
            g = dict(np.load(out)) if out.exists() else {}
            run_ensemble(O, g)
        elif a.startswith("mhd"):
            n, out = int(a[3:]), OUT3
            g = dict(np.load(out)) if out.exists() else {}
            run_mhd(O, n, g)
        else:
            n, out = int(a), OUT
            g = dict(np.load(out)) if out.exists() else {}
            run_size(O, n, g)
        np.savez_compressed(out, **g)
        print(f"wrote {out}")


if __name__ == "__main__":
    main()
