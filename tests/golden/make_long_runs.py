"""Generate tests/golden/long_rk4.npz: the 1000-step RK4 runs of the plain 2D solver
at 512^2 and 2048^2, computed by the FFTW-backed oracle.

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

    python tests/golden/make_long_runs.py [512] [2048]
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


def main() -> None:
    sizes = [int(a) for a in sys.argv[1:]] or [512, 2048]
    O = orc.load(fftw=True)
    assert O.is_fftw
    O.set_threads(8)
    g: dict[str, np.ndarray] = dict(np.load(OUT)) if OUT.exists() else {}
    for n in sizes:
        run_size(O, n, g)
        np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
