"""GPU tests of libtara's Fourier neural operator (tara_fno_*) against the CPU
oracle in PyTorch FP64: forward outputs, gradients of the MSE loss, the Adam
update and the batch gather, in FP32 mode (tight tolerances) and in the BF16
tensor-core mode (tolerances of BF16 operand rounding), at a small shape and at
the closure's production shape (128^2, 32 channels, 16 modes, 4 layers)."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2
from oracle import fno_oracle as fo

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SMALL = dict(h=32, w=32, ci=1, c=8, co=2, mx=6, my=8, layers=2, p=16, max_batch=8)


def _net(mode, **kw):
    cfg = tg.fno_default_config(**{**SMALL, **kw})
    cfg.mode = mode
    return tg.FNO(cfg)


def _data(net, B, seed):
    c = net.cfg
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, c.h, c.w, c.ci)).astype(np.float32)
    t = rng.standard_normal((B, c.h, c.w, c.co)).astype(np.float32)
    return x, t


def _dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()  # the library's streams do not wait on torch's stream
    return t


def _blocks(s: fo.FnoShape, g: np.ndarray) -> dict:
    out, o = {}, 0
    for name, sh in s.sizes():
        n = int(np.prod(sh))
        out[name] = g[o:o + n]
        o += n
    return out


def _forward_gpu(net, x, B):
    c = net.cfg
    xd = _dev(x)
    yd = torch.empty((B, c.h, c.w, c.co), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.forward(xd.data_ptr(), yd.data_ptr(), B)
    return yd.cpu().numpy()


@pytest.mark.parametrize("batch", [3, 6])  # per-mode GEMV (<= 4 samples) and tensor-core GEMM
@pytest.mark.parametrize("mode,tol", [(tg.FNO_FP32, 2e-6), (tg.FNO_BF16, 2e-2)])
def test_forward_matches_oracle(mode, tol, batch):
    with _net(mode) as net:
        s = fo.FnoShape.of(net.cfg)
        x, _ = _data(net, batch, 10)
        p = net.get_params()
        y = _forward_gpu(net, x, batch)
        ref = fo.forward(torch.tensor(p, dtype=torch.float64), torch.tensor(x, dtype=torch.float64), s)
        assert rel_l2(y, ref.numpy()) < tol


@pytest.mark.parametrize("mode,tol", [(tg.FNO_FP32, 2e-5), (tg.FNO_BF16, 4e-2)])
def test_gradients_match_oracle(mode, tol):
    with _net(mode) as net:
        s = fo.FnoShape.of(net.cfg)
        x, t = _data(net, 4, 11)
        p = net.get_params()
        xd, td = _dev(x), _dev(t)
        loss = net.train_step(xd.data_ptr(), td.data_ptr(), 4, lr=0.0)
        g = net.get_grads()
        ref_loss, ref_g = fo.loss_and_grad(p, x, t, s)
        assert abs(loss - ref_loss) < tol * ref_loss
        gb, rb = _blocks(s, g), _blocks(s, ref_g)
        for name in gb:
            assert rel_l2(gb[name], rb[name]) < tol, name
        cos = float(np.dot(g, ref_g) / (np.linalg.norm(g) * np.linalg.norm(ref_g)))
        assert cos > 1 - tol


def test_adam_update_matches_oracle():
    with _net(tg.FNO_FP32) as net:
        x, t = _data(net, 2, 12)
        xd, td = _dev(x), _dev(t)
        p0 = net.get_params().astype(np.float64)
        m = np.zeros_like(p0)
        v = np.zeros_like(p0)
        p = p0
        for step in (1, 2, 3):
            net.train_step(xd.data_ptr(), td.data_ptr(), 2, lr=0.0)  # gradients at the current params
            g = net.get_grads().astype(np.float64)
            net.train_step(xd.data_ptr(), td.data_ptr(), 2, lr=1e-3)  # same gradients, then the update
            p, m, v = fo.adam(p, g, m, v, step, 1e-3)
            got = net.get_params().astype(np.float64)
            assert np.max(np.abs(got - p)) < 1e-6, step
        assert net.adam_steps == 3


def test_indexed_batch_equals_contiguous_batch():
    with _net(tg.FNO_BF16) as net:
        x, t = _data(net, 4, 13)
        idx = np.array([3, 0, 2], np.int32)
        # (device tensors are bound to names: a temporary's memory could be reused)
        full_x, full_t, idx_d = _dev(x), _dev(t), _dev(idx)
        l1 = net.train_step(full_x.data_ptr(), full_t.data_ptr(), 3, idx_ptr=idx_d.data_ptr(), n_samples=4)
        g1 = net.get_grads()
        sub_x, sub_t = _dev(x[idx]), _dev(t[idx])
        l2 = net.train_step(sub_x.data_ptr(), sub_t.data_ptr(), 3)
        g2 = net.get_grads()
        assert l1 == l2
        assert np.array_equal(g1, g2)
        bad = _dev(np.array([4], np.int32))
        with pytest.raises(tg.TaraError):  # index 4 is outside a 4-sample dataset
            net.train_step(full_x.data_ptr(), full_t.data_ptr(), 1, idx_ptr=bad.data_ptr(), n_samples=4)


def test_production_shape_forward_bf16():
    cfg = tg.fno_default_config(max_batch=2)
    with tg.FNO(cfg) as net:
        assert (cfg.h, cfg.w, cfg.c, cfg.mx, cfg.my, cfg.layers) == (128, 128, 32, 16, 32, 4)
        s = fo.FnoShape.of(cfg)
        assert net.num_params == s.num_params()
        x = np.random.default_rng(14).standard_normal((2, 128, 128, 1)).astype(np.float32)
        y = _forward_gpu(net, x, 2)
        ref = fo.forward(torch.tensor(net.get_params(), dtype=torch.float64),
                         torch.tensor(x, dtype=torch.float64), s)
        assert rel_l2(y, ref.numpy()) < 2e-2


def test_training_reduces_loss():
    """A learnable target (a fixed random FNO's output) is fitted by Adam."""
    with _net(tg.FNO_BF16, seed=99) as teacher, _net(tg.FNO_BF16, seed=5) as net:
        x = np.random.default_rng(15).standard_normal((4, 32, 32, 1)).astype(np.float32)
        t = _forward_gpu(teacher, x, 4)
        xd, td = _dev(x), _dev(t)
        first = net.train_step(xd.data_ptr(), td.data_ptr(), 4, lr=0.0)
        for _ in range(300):
            net.train_step(xd.data_ptr(), td.data_ptr(), 4, lr=3e-3, want_loss=False)
        last = net.train_step(xd.data_ptr(), td.data_ptr(), 4, lr=0.0)
        assert last < 0.1 * first


CLOSURE_CH = dict(h=32, w=32, ci=6, c=32, co=2, mx=8, my=16, layers=2, p=128, max_batch=8)


@pytest.mark.parametrize("mode", [tg.FNO_BF16, tg.FNO_BF16_TMEM])
@pytest.mark.parametrize("batch", [2, 6])
def test_tensor_core_kernels_match_oracle(batch, mode):
    """BF16 modes at the closure's channel counts (6 -> 32 -> 128 -> 2), where the
    tall-skinny tensor-core GEMMs (pointwise mixing, head, input gradients; on
    mma.sync or on tcgen05 with tensor-memory accumulators) and the
    weight-gradient reductions (with the fused bias gradients) run."""
    cfg = tg.fno_default_config(**CLOSURE_CH)
    cfg.mode = mode
    with tg.FNO(cfg) as net:
        s = fo.FnoShape.of(cfg)
        x, t = _data(net, batch, 20 + batch)
        p = net.get_params()
        y = _forward_gpu(net, x, batch)
        ref = fo.forward(torch.tensor(p, dtype=torch.float64), torch.tensor(x, dtype=torch.float64), s)
        assert rel_l2(y, ref.numpy()) < 2e-2
        xd, td = _dev(x), _dev(t)
        loss = net.train_step(xd.data_ptr(), td.data_ptr(), batch, lr=0.0)
        g = net.get_grads()
        ref_loss, ref_g = fo.loss_and_grad(p, x, t, s)
        assert abs(loss - ref_loss) < 2e-2 * ref_loss
        gb, rb = _blocks(s, g), _blocks(s, ref_g)
        for name in gb:
            assert rel_l2(gb[name], rb[name]) < 4e-2, name
        cos = float(np.dot(g, ref_g) / (np.linalg.norm(g) * np.linalg.norm(ref_g)))
        assert cos > 0.996


def test_tcgen05_gemms_match_mma_sync():
    """The tcgen05 form of the channel GEMMs (TARA_FNO_BF16_TMEM) against the
    mma.sync form at the production shape (128^2, 6 -> 32 -> 128 -> 2, batch 8:
    1024 row tiles per GEMM, several per CTA): both multiply the same BF16-rounded
    operands with FP32 accumulation, so outputs, loss and gradients agree to
    FP32 summation-order differences."""
    cfg = tg.fno_default_config(ci=6, max_batch=8)
    with tg.FNO(cfg) as net:
        x = np.random.default_rng(31).standard_normal((8, 128, 128, 6)).astype(np.float32)
        t = np.random.default_rng(32).standard_normal((8, 128, 128, 2)).astype(np.float32)
        y0 = _forward_gpu(net, x, 8)
        xd, td = _dev(x), _dev(t)
        l0 = net.train_step(xd.data_ptr(), td.data_ptr(), 8, lr=0.0)
        g0 = net.get_grads()
        net.set_mode(tg.FNO_BF16_TMEM)
        y1 = _forward_gpu(net, x, 8)
        l1 = net.train_step(xd.data_ptr(), td.data_ptr(), 8, lr=0.0)
        g1 = net.get_grads()
        assert rel_l2(y1, y0) < 1e-5
        assert abs(l1 - l0) < 1e-5 * l0
        assert rel_l2(g1, g0) < 1e-4
        # training in the tcgen05 form: Adam steps keep the loss finite and decreasing
        for _ in range(20):
            net.train_step(xd.data_ptr(), td.data_ptr(), 8, lr=1e-3, want_loss=False)
        l2 = net.train_step(xd.data_ptr(), td.data_ptr(), 8, lr=0.0)
        assert np.isfinite(l2) and l2 < l1


@pytest.mark.parametrize("mode", [tg.FNO_BF16, tg.FNO_BF16_TMEM])
@pytest.mark.parametrize("kw,batches", [
    (dict(ci=6), (1, 3)),                       # the closure's network (p = 128, co = 2)
    (dict(ci=1, h=64, p=64, co=1), (2,)),       # 64 grid rows, a narrower projection
    (dict(ci=3, p=256, co=4, my=16, mx=8), (4,)),
])
def test_fused_inference_matches_layer_by_layer(mode, kw, batches):
    """The fused small-batch inference forward (lift + 2 launches per layer,
    tcgen05 pointwise and projection products) against the layer-by-layer
    forward of the training step on the same BF16-rounded operands, and against
    the FP64 oracle at BF16 tolerance.  The two forwards sum in different orders
    in FP32; where that moves an activation across a BF16 rounding boundary the
    next layer's operand differs by one BF16 unit (2^-8 relative), so they agree
    to about 1e-4, not to FP32 precision."""
    cfg = tg.fno_default_config(max_batch=4, **kw)
    cfg.mode = mode
    with tg.FNO(cfg) as net:
        s = fo.FnoShape.of(cfg)
        for B in batches:
            x = np.random.default_rng(40 + B).standard_normal((B, cfg.h, cfg.w, cfg.ci)).astype(np.float32)
            net.set_fused(True)
            y_fused = _forward_gpu(net, x, B)
            net.set_fused(False)
            y_layers = _forward_gpu(net, x, B)
            assert rel_l2(y_fused, y_layers) < 1e-3, B
            ref = fo.forward(torch.tensor(net.get_params(), dtype=torch.float64),
                             torch.tensor(x, dtype=torch.float64), s)
            assert rel_l2(y_fused, ref.numpy()) < 2e-2, B


@pytest.mark.parametrize("mode", [tg.FNO_BF16, tg.FNO_BF16_TMEM])
def test_tensor_core_dfts_at_production_shape(mode):
    """At the closure's network shape (W = 128, 32 channels, 16 kx modes) the
    truncated DFTs along x run as tcgen05 products with split-BF16 operands in
    the BF16 modes (forward and the adjoints of the backward pass): the
    layer-by-layer forward, the loss and every parameter block's gradient
    against the FP64 oracle at the BF16 tolerances, at batch 2 and 6 (the
    per-mode GEMV and the batched mixing GEMM)."""
    cfg = tg.fno_default_config(ci=6, max_batch=6)
    cfg.mode = mode
    with tg.FNO(cfg) as net:
        net.set_fused(False)
        s = fo.FnoShape.of(cfg)
        p = net.get_params()
        for B in (2, 6):
            x, t = _data(net, B, 60 + B)
            y = _forward_gpu(net, x, B)
            ref = fo.forward(torch.tensor(p, dtype=torch.float64), torch.tensor(x, dtype=torch.float64), s)
            assert rel_l2(y, ref.numpy()) < 2e-2, B
            xd, td = _dev(x), _dev(t)
            loss = net.train_step(xd.data_ptr(), td.data_ptr(), B, lr=0.0)
            g = net.get_grads()
            ref_loss, ref_g = fo.loss_and_grad(p, x, t, s)
            assert abs(loss - ref_loss) < 2e-2 * ref_loss, B
            gb, rb = _blocks(s, g), _blocks(s, ref_g)
            for name in gb:
                assert rel_l2(gb[name], rb[name]) < 4e-2, (B, name)
            cos = float(np.dot(g, ref_g) / (np.linalg.norm(g) * np.linalg.norm(ref_g)))
            assert cos > 0.996, B
