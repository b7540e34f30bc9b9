"""CPU tests of the learned-closure oracle (oracle/fno_oracle.py): the rfft2
form of the spectral convolution equals its explicit-sum restatement, autograd
gradients equal finite differences, and the box filter / shell spectrum keep
their defining identities.  These pin the oracle the GPU tests rely on."""
from __future__ import annotations

import numpy as np
import torch

from oracle import fno_oracle as fo

SMALL = fo.FnoShape(h=16, w=12, ci=1, c=3, co=2, mx=4, my=6, layers=2, p=5)


def test_spectral_conv_matches_explicit_sums():
    g = torch.Generator().manual_seed(1)
    s = SMALL
    v = torch.randn(2, s.h, s.w, s.c, generator=g, dtype=torch.float64)
    R = torch.randn(s.my, s.mx, s.c, s.c, 2, generator=g, dtype=torch.float64)
    a = fo.spectral_conv(v, R, s)
    b = fo.spectral_conv_dft(v, R, s)
    assert torch.max(torch.abs(a - b)) < 1e-12 * torch.max(torch.abs(b))


def test_forward_forms_agree():
    rng = np.random.default_rng(2)
    s = SMALL
    p = torch.tensor(rng.standard_normal(s.num_params()) * 0.3)
    x = torch.tensor(rng.standard_normal((2, s.h, s.w, s.ci)))
    a = fo.forward(p, x, s)
    b = fo.forward(p, x, s, dft=True)
    assert a.shape == (2, s.h, s.w, s.co)
    assert torch.max(torch.abs(a - b)) < 1e-11


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    s = SMALL
    p = rng.standard_normal(s.num_params()) * 0.3
    x = rng.standard_normal((2, s.h, s.w, s.ci))
    t = rng.standard_normal((2, s.h, s.w, s.co))
    _, g = fo.loss_and_grad(p, x, t, s)
    for i in rng.choice(p.size, 12, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        lp, _ = fo.loss_and_grad(p + e, x, t, s)
        lm, _ = fo.loss_and_grad(p - e, x, t, s)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_adam_first_step_moves_by_lr():
    p = np.array([1.0, -2.0, 3.0])
    g = np.array([0.5, -0.1, 0.0])
    q, m, v = fo.adam(p, g, np.zeros(3), np.zeros(3), 1, 1e-3)
    # the first bias-corrected step is lr * sign(g) (up to eps)
    assert np.allclose(q - p, -1e-3 * np.sign(g), atol=1e-10)


def test_velocity_of_single_mode():
    n = 32
    x = 2 * np.pi * np.arange(n) / n
    omega = np.cos(3 * x)[None, :].repeat(n, 0)  # w = cos(3x): psi = cos(3x)/9
    u, v = fo.velocity(omega)
    assert np.max(np.abs(u)) < 1e-14
    assert np.allclose(v, np.sin(3 * x)[None, :] / 3.0, atol=1e-14)


def test_box_filter_identities():
    rng = np.random.default_rng(4)
    w = rng.standard_normal((32, 32))
    wb, flux = fo.box_filter(w, 1)
    assert np.allclose(wb, w) and np.max(np.abs(flux)) < 1e-12
    wb4, flux4 = fo.box_filter(w, 4)
    assert wb4.shape == (8, 8) and flux4.shape == (8, 8, 2)
    assert abs(wb4.mean() - w.mean()) < 1e-14


def test_shell_spectrum_sums_to_energy():
    rng = np.random.default_rng(5)
    wk = np.fft.rfft2(rng.standard_normal((64, 64)))
    wk[0, 0] = 0.0
    wk[32, :] = 0.0  # no Nyquist modes: their derivatives have no real field
    wk[:, 32] = 0.0
    w = np.fft.irfft2(wk, s=(64, 64))
    u, v = fo.velocity(w)
    E = fo.shell_spectrum(w, 64)  # kmax >= sqrt(2)*32 covers every mode
    assert abs(E.sum() - 0.5 * np.mean(u * u + v * v)) < 1e-12 * E.sum()
