"""Lagrangian passive particles of the plain driver (src/main2csh.f95:187-273):
the driver's random-number generator (CPU known-answer test) and the GPU
interpolation + Euler + wrap step against the oracle, including particles on
the last cell column and row and on the box edge."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

PI = np.pi


def test_park_miller_known_answer():
    # Park & Miller (1988): from seed 1 the 10000th state of the minimal standard is 1043618065
    _, state = tg.park_miller(10000, 1)
    assert state == 1043618065
    r, _ = tg.park_miller(3, 1)
    assert r[0] == np.float32(16384 * 2.0**-31)  # (16807 - 1) with the low 9 bits cleared


@pytest.mark.gpu
def test_particles_match_oracle(oracle):
    n, lx, ly = 64, 2 * PI * 2.0, 2 * PI * 1.5  # rectangular box with the driver's true pi
    rng = np.random.default_rng(7)
    xp = rng.uniform(0, lx, 500)
    yp = rng.uniform(0, ly, 500)
    dx, dy = lx / n, ly / n
    edge_x = [lx, lx - 1e-9, 1e-12, (n - 1) * dx + 0.5 * dx, 0.5 * dx, lx]
    edge_y = [ly, 0.5 * dy, ly - 1e-9, (n - 1) * dy + 0.25 * dy, ly, 1e-12]
    xp = np.concatenate([xp, edge_x])
    yp = np.concatenate([yp, edge_y])
    with tg.Solver2D(n, nu=1e-3, dt=2e-3) as s, tg.Particles(s, xp, yp, lx, ly) as p:
        s.init_random(4.0, 0.5, 31)
        ox, oy = xp.copy(), yp.copy()
        for _ in range(6):
            s.step(1)
            p.advance(0.05)  # large steps so that particles cross cells and the box edge
            w = s.get_state()
            vx, vy = oracle.driver_velocity(w, lx, ly)
            ox, oy = oracle.particles_step(vx, vy, ox, oy, lx, ly, 0.05)
            gx, gy = p.positions()
            assert np.abs(gx - ox).max() < 1e-11 * lx
            assert np.abs(gy - oy).max() < 1e-11 * ly
        assert np.all((gx > 0) & (gx <= lx)) and np.all((gy > 0) & (gy <= ly))
        assert rel_l2(gx, xp) > 1e-3  # the particles moved
