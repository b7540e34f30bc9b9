"""CPU: the twiddle tables the transforms read (tara_twiddle_table, the host code
that fills them), checked against their definition and run through a numpy
model of the device's stage sequence (fft.cuh) that indexes them exactly as the
kernels do:

  FP64, even log2 n   untwiddled radix-4 stage, then ratio-form radix-4 stages
                      at Ns = 4, 16, ... (dft4_tw_ratio; entries (tau, c) and
                      (tau3, c3 / c1), tau = s / c)
  FP64, odd log2 n    untwiddled 8-point DFT, then ratio-form radix-4 stages at
                      Ns = 8, 32, ... (fft_slot_m8, its own table region)
  FP32 tables         the plain twiddles: radix-4 stages with complex twiddles,
                      then for odd log2 n a radix-2 stage reading W^j (W^(n-j)
                      for the inverse)

The models compute in float64 from the library's tables and must reproduce
numpy's FFT to 1e-14 (relative L2), forward and inverse."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


def _lg(n):
    return n.bit_length() - 1


def stage_span(n):  # tw_stage_span
    return (1 << (2 * (_lg(n) // 2))) - 4


def r8_span(n):  # the radix-8 path's tables (fft.cuh r8_* helpers)
    lg = _lg(n)
    s8 = lg // 3 - 1 if (lg % 3 == 1 and lg >= 4) else lg // 3
    s4 = 2 if lg % 3 == 1 else 1 if lg % 3 == 2 else 0
    radix = [8] * s8 + [4] * s4
    ns = [1]
    for r in radix[:-1]:
        ns.append(ns[-1] * r)
    return sum((4 if r == 8 else 3) * m for r, m in zip(radix[1:], ns[1:]))


def m8_base(n):
    return n + 2 * stage_span(n) + 2 * r8_span(n)


def m8_span(n):
    return 8 * ((1 << (_lg(n) - 3)) - 1) if (_lg(n) & 1) and n >= 32 else 0


def W(n, e):
    return np.exp(-2j * np.pi * (np.asarray(e) % n) / n)


def ratio_butterfly(v, e1, e2, e3, inv):
    """dft4_tw_ratio on arrays of butterflies; e_r = (tau, c or rho) rows."""
    t1, c1 = e1[:, 0], e1[:, 1]
    t2, c2 = e2[:, 0], e2[:, 1]
    t3, rho = e3[:, 0], e3[:, 1]
    z1 = v[1] * (1 + 1j * t1)
    z2 = v[2] * (1 + 1j * t2)
    z3 = v[3] * (1 + 1j * t3)
    a0, a1 = v[0] + c2 * z2, v[0] - c2 * z2
    b, d = z1 + rho * z3, z1 - rho * z3
    mi = 1j if inv else -1j
    return [a0 + c1 * b, a1 + mi * c1 * d, a0 - c1 * b, a1 - mi * c1 * d]


def plain_butterfly(v, w1, w2, w3, inv):
    t = [v[0], w1 * v[1], w2 * v[2], w3 * v[3]]
    mi = 1j if inv else -1j
    return [t[0] + t[1] + t[2] + t[3], t[0] + mi * t[1] - t[2] - mi * t[3],
            t[0] - t[1] + t[2] - t[3], t[0] - mi * t[1] - t[2] + mi * t[3]]


def radix4_stage(buf, n, ns, entries, inv, ratio):
    """One Stockham radix-4 stage: butterfly j reads buf[j + r n/4], writes
    out[(j - k) 4 + k + r ns], k = j mod ns; entries(r, k) -> table rows."""
    q = n // 4
    j = np.arange(q)
    k = j % ns
    v = [buf[j + r * q] for r in range(4)]
    if ns == 1:
        y = plain_butterfly(v, 1, 1, 1, inv)
    elif ratio:
        y = ratio_butterfly(v, entries(1, k), entries(2, k), entries(3, k), inv)
    else:
        e = [entries(r, k) for r in (1, 2, 3)]
        y = plain_butterfly(v, *[x[:, 0] + 1j * x[:, 1] for x in e], inv)
    out = np.empty_like(buf)
    base = (j - k) * 4 + k
    for r in range(4):
        out[base + r * ns] = y[r]
    return out


def model_fp64(x, tab, inv):
    n = len(x)
    lg = _lg(n)
    buf = x.astype(np.complex128)
    if lg & 1:
        b8 = n // 8
        j = np.arange(b8)
        v = np.stack([buf[j + r * b8] for r in range(8)])
        f8 = np.exp((2j if inv else -2j) * np.pi * np.outer(np.arange(8), np.arange(8)) / 8)
        out = np.empty_like(buf)
        for qq in range(8):
            out[8 * j + qq] = f8[qq] @ v
        buf = out
        start = m8_base(n) + (m8_span(n) if inv else 0)
        ns = 8
        while ns < n:
            base = start + ns - 8
            buf = radix4_stage(buf, n, ns, lambda r, k, b=base, s=ns: tab[b + (r - 1) * s + k], inv, True)
            ns *= 4
    else:
        start = n + (stage_span(n) if inv else 0)
        ns = 1
        while ns < n:
            base = start + ns - 4
            buf = radix4_stage(buf, n, ns, lambda r, k, b=base, s=ns: tab[b + (r - 1) * s + k], inv, True)
            ns *= 4
    return buf


def model_plain(x, tab, inv):
    n = len(x)
    buf = x.astype(np.complex128)
    start = n + (stage_span(n) if inv else 0)
    ns = 1
    while 4 * ns <= n:
        base = start + ns - 4
        buf = radix4_stage(buf, n, ns, lambda r, k, b=base, s=ns: tab[b + (r - 1) * s + k], inv, False)
        ns *= 4
    if ns < n:  # final radix-2 stage, Ns = n/2
        h = n // 2
        j = np.arange(h)
        idx = (n - j) % n if inv else j
        w = tab[idx, 0] + 1j * tab[idx, 1]
        a, c = buf[j].copy(), buf[j + h].copy()
        buf[j], buf[j + h] = a + w * c, a - w * c
    return buf


@pytest.mark.parametrize("n", SIZES)
def test_tables_match_their_definition(n):
    f64 = tg.twiddle_table(n, tg.PREC_FP64)
    f32 = tg.twiddle_table(n, tg.PREC_FP32)
    assert f64.shape == f32.shape == (m8_base(n) + 2 * m8_span(n), 2)
    w = W(n, np.arange(n))
    assert np.abs(f64[:n, 0] + 1j * f64[:n, 1] - w).max() < 1e-15
    assert np.array_equal(f64[:n], f32[:n])
    # the conjugate twiddle sits at the mirrored index, exactly
    assert np.array_equal(f64[1:n, 0], f64[n - 1:0:-1, 0]) and np.array_equal(f64[1:n, 1], -f64[n - 1:0:-1, 1])
    for start, span, first in ((n, stage_span(n), 4), (m8_base(n), m8_span(n), 8)):
        for d, inv in ((0, False), (1, True)):
            ns = first
            while ns - first < span:
                k = np.arange(ns)
                base = start + d * span + ns - first
                c = [None]
                for r in (1, 2, 3):
                    wr = W(n, r * k * (n // (4 * ns)))
                    if inv:
                        wr = np.conj(wr)
                    plain = f32[base + (r - 1) * ns + k]
                    assert np.abs(plain[:, 0] + 1j * plain[:, 1] - wr).max() < 1e-15
                    cr = np.where(plain[:, 0] == 0.0, 2.0 ** -256, plain[:, 0])
                    c.append(cr)
                    ent = f64[base + (r - 1) * ns + k]
                    assert np.array_equal(ent[:, 0], plain[:, 1] / cr)  # tau = s / c
                    assert np.array_equal(ent[:, 1], cr if r < 3 else cr / c[1])  # c, or c3 / c1
                ns *= 4


def test_quarter_turn_cosine_is_a_power_of_two():
    """w2 at k = Ns/2 is the quarter turn: its cosine is stored as 2^-256 and its
    tau as s 2^256, so c tau = s holds exactly."""
    n = 64
    f64 = tg.twiddle_table(n, tg.PREC_FP64)
    ns = 16
    e = f64[n + ns - 4 + ns + ns // 2]  # forward, r = 2, k = Ns/2
    assert e[1] == 2.0 ** -256 and e[0] * e[1] == -1.0


@pytest.mark.parametrize("n", SIZES)
def test_device_stage_models_reproduce_the_dft(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f64 = tg.twiddle_table(n, tg.PREC_FP64)
    f32 = tg.twiddle_table(n, tg.PREC_FP32)
    fwd, bwd = np.fft.fft(x), np.fft.ifft(x) * n
    assert rel_l2(model_fp64(x, f64, False), fwd) < 1e-14
    assert rel_l2(model_fp64(x, f64, True), bwd) < 1e-14
    assert rel_l2(model_plain(x, f32, False), fwd) < 1e-14
    assert rel_l2(model_plain(x, f32, True), bwd) < 1e-14


def test_table_export_validates_arguments():
    import ctypes

    cnt = ctypes.c_int()
    for n, prec in ((48, tg.PREC_FP64), (8192, tg.PREC_FP64), (64, tg.PREC_DF64)):
        assert tg.lib().tara_twiddle_table(n, prec, None, 0, ctypes.byref(cnt)) == tg.TARA_ERR_ARGS
    buf = np.zeros((4, 2))
    rc = tg.lib().tara_twiddle_table(64, tg.PREC_FP64, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4,
                                     ctypes.byref(cnt))
    assert rc == tg.TARA_ERR_ARGS and cnt.value > 4 and not buf.any()


# ---- the 8-point DFT of fft.cuh, single lane (dft8) and split over a lane pair
C8 = 0.70710678118654752440


def _mul_w4(t, inv):  # exact: a swap and a sign
    return (-t[1], t[0]) if inv else (t[1], -t[0])


def _pair_1(a, b):
    return (a[0] + b[0], a[1] + b[1]), (a[0] - b[0], a[1] - b[1])


def _pair_w4(a, b, inv):
    return _pair_1(a, _mul_w4(b, inv))


def _pair_w8(a, b, inv, e):
    x, y = b
    if not inv:
        p, q = (x + y, y - x) if e == 1 else (y - x, -(x + y))
    else:
        p, q = (x - y, x + y) if e == 1 else (-(x + y), x - y)
    return (a[0] + C8 * p, a[1] + C8 * q), (a[0] - C8 * p, a[1] - C8 * q)


def _dft8(v, inv):
    v = list(v)
    for i in range(4):
        v[i], v[i + 4] = _pair_1(v[i], v[i + 4])
    v[0], v[2] = _pair_1(v[0], v[2])
    v[1], v[3] = _pair_1(v[1], v[3])
    v[4], v[6] = _pair_w4(v[4], v[6], inv)
    v[5], v[7] = _pair_w4(v[5], v[7], inv)
    v[0], v[1] = _pair_1(v[0], v[1])
    v[2], v[3] = _pair_w4(v[2], v[3], inv)
    v[4], v[5] = _pair_w8(v[4], v[5], inv, 1)
    v[6], v[7] = _pair_w8(v[6], v[7], inv, 3)
    out = [None] * 8
    for i, q in enumerate((0, 4, 2, 6, 1, 5, 3, 7)):
        out[q] = v[i]
    return out


def _dft8_lane_pair(v, inv):
    lanes = []
    for odd in (0, 1):
        u = [v[2 * i + odd] for i in range(4)]
        u[0], u[2] = _pair_1(u[0], u[2])
        u[1], u[3] = _pair_1(u[1], u[3])
        u[0], u[1] = _pair_1(u[0], u[1])
        u[2], u[3] = _pair_w4(u[2], u[3], inv)
        lanes.append(u)
    out = [None] * 8
    for odd in (0, 1):
        u, w = lanes[odd], lanes[1 - odd]
        r0, r1 = (w[1], w[3]) if odd else (w[0], w[2])  # what the partner lane sends
        x0 = r0 if odd else u[0]
        x1 = _mul_w4(u[1], inv) if odd else r0
        x4 = r1 if odd else u[2]
        x5 = _mul_w4(u[3], inv) if odd else r1
        x0, x1 = _pair_1(x0, x1)
        x4, x5 = _pair_w8(x4, x5, inv, 1)
        o = 2 if odd else 0
        out[o], out[o + 4], out[o + 1], out[o + 5] = x0, x1, x4, x5
    return out


@pytest.mark.parametrize("inv", [False, True])
def test_lane_pair_8point_dft_gives_the_single_lane_bits(inv):
    """fft_slot_m8's lane-pair form runs dft8's pairs on the same operands: the odd
    lane's (x2, W4 x3) and (x6, W4 x7) pairs reproduce pair_w4 and pair_w8<3> bit
    for bit, and both equal the DFT to rounding."""
    rng = np.random.default_rng(8 + inv)
    for _ in range(200):
        z = rng.standard_normal((8, 2)) * 10.0 ** rng.integers(-5, 6, size=(8, 1))
        v = [tuple(r) for r in z]
        a, b = _dft8(v, inv), _dft8_lane_pair(v, inv)
        assert all(p == q for p, q in zip(a, b))
        x = z[:, 0] + 1j * z[:, 1]
        ref = np.fft.ifft(x) * 8 if inv else np.fft.fft(x)
        got = np.array([complex(*t) for t in a])
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(x).sum()
