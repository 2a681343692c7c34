"""The learned coarse-slice closure on the GPU: its forward pass and its
gradient (tensor-core and CUDA-core kernels, bf16 weights and activations,
FP32 accumulation) against the float64 CPU oracle (oracle/closure_oracle.py)
computed with the same bf16 rounding points, and the optimiser reducing the
loss."""
import numpy as np
import pytest

from oracle import closure_oracle as CO

pytestmark = pytest.mark.gpu


def _waves(seed, B, H, W):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W]
    base = np.exp(1j * (2 * np.pi * (3 * x / W + 2 * y / H)))
    c = (base[None] * (1 + 0.3 * rng.standard_normal((B, H, W)))
         + 0.2j * rng.standard_normal((B, H, W))).astype(np.complex64)
    f = (c + 0.05 * (rng.standard_normal((B, H, W)) + 1j * rng.standard_normal((B, H, W)))).astype(np.complex64)
    return c, f


def _layer_slices():
    offs = np.cumsum([0] + [9 * co * ci * 2 + co * 2 for ci, co in CO.LAYERS])
    return [slice(offs[i], offs[i + 1]) for i in range(6)]


def test_closure_forward_matches_oracle(ctx):
    from multislice_gb300.api import Closure
    net = Closure(ctx, seed=7)
    p = CO.init_params(11, scale_last=1.0)
    net.set_params(p)
    c, _ = _waves(1, 2, 6, 128)
    got = net.apply(c.copy())
    ref, _, _ = CO.forward(p, c, bf=True)
    d_got, d_ref = got - c, ref - c
    assert np.linalg.norm(d_ref) > 0.1 * np.linalg.norm(c)
    assert np.linalg.norm(d_got - d_ref) / np.linalg.norm(d_ref) < 1e-3
    net.close()


def test_closure_gradient_matches_oracle(ctx):
    from multislice_gb300.api import Closure
    net = Closure(ctx, seed=7)
    p = CO.init_params(12, scale_last=1.0)
    net.set_params(p)
    c, f = _waves(2, 2, 6, 128)
    loss, g = net.gradients(c, f)
    ref_loss, ref_g = CO.gradient(p, c, f, bf=True)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    for l, sl in enumerate(_layer_slices()):
        err = np.linalg.norm(g[sl] - ref_g[sl]) / np.linalg.norm(ref_g[sl])
        assert err < 2e-2, (l, err)
    net.close()


def test_closure_training_reduces_loss(ctx):
    from multislice_gb300.api import Closure
    net = Closure(ctx, seed=3)
    c, _ = _waves(4, 4, 8, 128)
    # a target the network can represent: a local linear map of the coarse wave
    f = (c + 0.05 * np.roll(c, 1, axis=2) + 0.03j * c).astype(np.complex64)
    first = net.train_step(c, f, 3e-3)
    for _ in range(100):
        last = net.train_step(c, f, 3e-3)
    assert last < 0.2 * first, (first, last)
    # the trained parameters leave the library and come back unchanged
    p = net.get_params()
    net2 = Closure(ctx, seed=99)
    net2.set_params(p)
    np.testing.assert_array_equal(net2.apply(c.copy()), net.apply(c.copy()))
    net.close()
    net2.close()


def test_closure_gain_on_held_out_srtio3_probes(ctx):
    """Trained on pairs the library makes (SrTiO3, 4x thicker slices), the closure
    brings held-out coarse-slice exit waves closer to the fine-slice ones than the
    coarse waves alone -- the gain over the method without it."""
    import torch

    from multislice_gb300 import closure as CL
    from multislice_gb300.api import Closure
    coarse, fine = CL.make_pairs(ctx, 192, seed=5, nconfig=4)
    tr_c, tr_f = coarse[:128].contiguous(), fine[:128].contiguous()
    va_c, va_f = coarse[128:].contiguous(), fine[128:].contiguous()
    net = Closure(ctx, seed=1)
    e_coarse, e_before = CL.evaluate(net, va_c, va_f)
    assert e_coarse > 1e-3                       # thicker slices do change the wave
    hist = CL.train(ctx, net, tr_c, tr_f, steps=300, batch=8, lr=2e-3, lr_final=2e-4, seed=2)
    assert hist[-1] < hist[0]
    e_coarse2, e_after = CL.evaluate(net, va_c, va_f)
    assert e_coarse2 == e_coarse
    assert e_after < 0.9 * e_coarse, (e_coarse, e_after)
    net.close()
    del coarse, fine
    torch.cuda.empty_cache()
