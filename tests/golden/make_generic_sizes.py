"""Generate tests/golden/generic_sizes.npz, computed by the FFTW-backed oracle,
for the grid sizes the reference accepts beyond powers of two (FFTW transforms
any length; the GPU takes even lengths with factors 2, 3, 5, 7 on its
mixed-radix path):

  s96   96 x 96, the reference's screen-free shear-layer initial vorticity
        (src/main2csh.f95:70-96, W0 = 25, m0 = 2, d = 3/128 of the default
        input.ini), its plain right-hand side (src/derive2csh.f95:19-145) and
        the state after 500 AB2 steps, nu = 0.01, dt = 1e-4 (src/ab2csh.f95);
  r48x80  48 x 80 (Nx x Ny), seeded random-phase vorticity (E(k) ~ k^4
        exp(-(k/4)^2), energy 0.5, seed 7), its plain right-hand side and the
        state after 200 classic RK4 steps, nu = 1e-3, dt = 1e-3;
  r56x84  56 x 84 (Nx x Ny, both with a factor 7), seeded random-phase
        vorticity (k0 = 5, energy 0.5, seed 11), its plain right-hand side and
        the state after 100 classic RK4 steps, nu = 1e-3, dt = 1e-3.

Every transform goes through FFTW 3.3.9 compiled from the reference's vendored
sources (oracle/_ref).  Run from the repository root:

    python tests/golden/make_generic_sizes.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as ob  # noqa: E402


def main():
    f = ob.load(fftw=True)
    out = {}
    w = f.r2c(f.ic_shear(96, 96))  # the driver's omegak = r2c(omega) (src/main2csh.f95:98-100)
    out["s96_w0"] = w
    out["s96_rhs"] = f.derive2csh(w, 0.01)
    out["s96_w500"] = f.run(w, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=500)[0]
    w = f.ic_random(48, 80, 4.0, 0.5, 7)
    out["r48x80_w0"] = w
    out["r48x80_rhs"] = f.derive2csh(w, 1e-3)
    out["r48x80_w200"] = f.run(w, rhs=0, scheme=1, nu=1e-3, dt=1e-3, steps=200)[0]
    w = f.ic_random(56, 84, 5.0, 0.5, 11)
    out["r56x84_w0"] = w
    out["r56x84_rhs"] = f.derive2csh(w, 1e-3)
    out["r56x84_w100"] = f.run(w, rhs=0, scheme=1, nu=1e-3, dt=1e-3, steps=100)[0]
    np.savez_compressed(ROOT / "tests" / "golden" / "generic_sizes.npz", **out)
    for k, v in out.items():
        print(k, v.shape, float(np.linalg.norm(v)))


if __name__ == "__main__":
    main()
