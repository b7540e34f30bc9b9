"""CPU oracle of the learned closure -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's checks import this
module, as the oracle of libtara's Fourier neural operator (tara_fno_*) and of
its closure pieces (box filter, shell spectrum).  Nothing here runs on the
product path.

The network has no counterpart in the reference (TARA has no learned model);
this file states its definition in PyTorch FP64 on the CPU in the standard
Fourier-neural-operator form (Li et al., "Fourier Neural Operator for
Parametric PDEs", ICLR 2021): rfft2, keep the low modes, per-mode complex
channel mixing, irfft2.  ``spectral_conv_dft`` restates the same operator as
explicit sums of complex exponentials, which pins the rfft2 form (checked by the
CPU tests together with finite differences of the autograd gradients).

Parameter layout (a flat FP32/FP64 vector, as in include/tara.h):
Pw (ci x c), Pb (c); per layer R (my x mx x c x c complex, interleaved), W (c x c),
b (c); Q1 (c x p), q1 (p), Q2 (p x co), q2 (co).  Row index j of R is ky mod my.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch


@dataclass
class FnoShape:
    h: int = 128
    w: int = 128
    ci: int = 1
    c: int = 32
    co: int = 2
    mx: int = 16
    my: int = 32
    layers: int = 4
    p: int = 128

    @classmethod
    def of(cls, cfg) -> "FnoShape":
        return cls(*(int(getattr(cfg, k)) for k in ("h", "w", "ci", "c", "co", "mx", "my", "layers", "p")))

    def sizes(self):
        s = [("Pw", (self.ci, self.c)), ("Pb", (self.c,))]
        for l in range(self.layers):
            s += [(f"R{l}", (self.my, self.mx, self.c, self.c, 2)), (f"W{l}", (self.c, self.c)),
                  (f"b{l}", (self.c,))]
        s += [("Q1", (self.c, self.p)), ("q1", (self.p,)), ("Q2", (self.p, self.co)), ("q2", (self.co,))]
        return s

    def num_params(self) -> int:
        return sum(int(np.prod(sh)) for _, sh in self.sizes())


def unpack(flat: torch.Tensor, s: FnoShape) -> dict:
    out, o = {}, 0
    for name, sh in s.sizes():
        n = int(np.prod(sh))
        out[name] = flat[o:o + n].reshape(sh)
        o += n
    assert o == flat.numel()
    return out


def _rows(s: FnoShape):
    """FFT row of each R index j: ky = j (j < my/2) or j - my."""
    return [j if j < s.my // 2 else s.h + j - s.my for j in range(s.my)]


def spectral_conv(v: torch.Tensor, R: torch.Tensor, s: FnoShape) -> torch.Tensor:
    """v (B, H, W, C) real -> (B, H, W, C): irfft2 of the mode-mixed rfft2."""
    X = torch.fft.rfft2(v.permute(0, 3, 1, 2))  # (B, C, H, W/2+1)
    Rc = torch.complex(R[..., 0], R[..., 1])    # (my, mx, C, C)
    out = torch.zeros(v.shape[0], s.c, s.h, s.w // 2 + 1, dtype=X.dtype)
    rows = _rows(s)
    Xs = X[:, :, rows, :s.mx]                   # (B, C, my, mx)
    out[:, :, rows, :s.mx] = torch.einsum("bcjk,jkco->bojk", Xs, Rc)
    return torch.fft.irfft2(out, s=(s.h, s.w)).permute(0, 2, 3, 1)


def spectral_conv_dft(v: torch.Tensor, R: torch.Tensor, s: FnoShape) -> torch.Tensor:
    """The same operator as explicit sums: X(ky,kx) = sum_{y,x} v e^{-i(kx x 2pi/W + ky y 2pi/H)},
    Y = X R, out = (1/HW) sum_{ky,kx} w_kx Re(Y e^{+i(...)}), w_0 = 1, w_kx = 2 (kx >= 1)."""
    B, H, W, C = v.shape
    ky = torch.tensor([j if j < s.my // 2 else j - s.my for j in range(s.my)], dtype=torch.float64)
    kx = torch.arange(s.mx, dtype=torch.float64)
    yy = torch.arange(H, dtype=torch.float64)
    xx = torch.arange(W, dtype=torch.float64)
    ey = torch.exp(-2j * np.pi * torch.outer(ky, yy) / H)   # (my, H)
    ex = torch.exp(-2j * np.pi * torch.outer(kx, xx) / W)   # (mx, W)
    vc = v.to(torch.complex128)
    X = torch.einsum("jy,kx,byxc->bjkc", ey, ex, vc)
    Y = torch.einsum("bjkc,jkco->bjko", X, torch.complex(R[..., 0], R[..., 1]))
    wk = torch.full((s.mx,), 2.0, dtype=torch.float64)
    wk[0] = 1.0
    Yw = Y * wk[None, None, :, None]
    out = torch.einsum("jy,kx,bjko->byxo", ey.conj(), ex.conj(), Yw).real / (H * W)
    return out


def forward(flat: torch.Tensor, x: torch.Tensor, s: FnoShape, dft: bool = False) -> torch.Tensor:
    """x (B, H, W, ci) -> y (B, H, W, co), FP64."""
    P = unpack(flat, s)
    gelu = torch.nn.functional.gelu
    v = x @ P["Pw"] + P["Pb"]
    conv = spectral_conv_dft if dft else spectral_conv
    for l in range(s.layers):
        z = conv(v, P[f"R{l}"], s) + v @ P[f"W{l}"] + P[f"b{l}"]
        v = gelu(z) if l < s.layers - 1 else z
    h = gelu(v @ P["Q1"] + P["q1"])
    return h @ P["Q2"] + P["q2"]


def loss_and_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray, s: FnoShape):
    """mean((y - t)^2) and its gradient with respect to the flat parameters, FP64."""
    flat = torch.tensor(np.asarray(params, np.float64), requires_grad=True)
    y = forward(flat, torch.tensor(np.asarray(x, np.float64)), s)
    loss = torch.mean((y - torch.tensor(np.asarray(t, np.float64))) ** 2)
    loss.backward()
    return float(loss.detach()), flat.grad.numpy().copy()


def adam(params, grad, m, v, step: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam update (Kingma & Ba 2015), FP64; returns (p, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return params - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


# ---------------------------------------------------------------------------
# closure pieces
# ---------------------------------------------------------------------------
def velocity(omega: np.ndarray):
    """u = d psi/dy, v = -d psi/dx with -lap psi = omega on the 2pi-periodic grid (y rows, x columns),
    integer wavenumbers; the mean mode of psi is zero and the Nyquist modes (kx = nx/2 or
    ky = -ny/2) contribute nothing.  (u_x = i ky psi_hat, u_y = -i kx psi_hat.)"""
    ny, nx = omega.shape
    w = np.fft.rfft2(omega)
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    kx = np.arange(nx // 2 + 1)[None, :]
    k2 = kx * kx + ky * ky
    k2[0, 0] = 1.0
    psi = w / k2
    psi[0, 0] = 0.0
    psi[ny // 2, :] = 0.0  # no odd derivative of the Nyquist modes
    psi[:, nx // 2] = 0.0
    return np.fft.irfft2(1j * ky * psi, s=omega.shape), np.fft.irfft2(-1j * kx * psi, s=omega.shape)


def box_filter(omega: np.ndarray, f: int):
    """Block means over f x f cells: omega_bar and the subgrid flux
    (bar(u w) - bar(u) bar(w), bar(v w) - bar(v) bar(w)) as (ny/f, nx/f, 2)."""
    u, v = velocity(omega)
    ny, nx = omega.shape

    def bar(a):
        return a.reshape(ny // f, f, nx // f, f).mean(axis=(1, 3))

    wb, ub, vb = bar(omega), bar(u), bar(v)
    flux = np.stack([bar(u * omega) - ub * wb, bar(v * omega) - vb * wb], axis=-1)
    return wb, flux


def shell_spectrum(omega: np.ndarray, kmax: int) -> np.ndarray:
    """E[k] = sum over round(|k|) = k of 1/2 |u_hat|^2 / (NxNy)^2 (full spectrum), k = 0..kmax."""
    ny, nx = omega.shape
    w = np.fft.fft2(omega)
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    kx = np.fft.fftfreq(nx, 1.0 / nx)[None, :]
    k2 = kx * kx + ky * ky
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    e = 0.5 * np.abs(w) ** 2 * inv / (nx * ny) ** 2
    shell = np.rint(np.sqrt(k2)).astype(int)
    out = np.zeros(kmax + 1)
    m = shell <= kmax
    np.add.at(out, shell[m], e[m])
    return out
