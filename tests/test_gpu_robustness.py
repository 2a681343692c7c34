"""Robustness on the GPU without provoking a fault: outputs written into the
middle of NaN-poisoned device buffers leave the poison around them untouched,
and a context memory cap turns an oversized request into MSL_E_NOMEM (an
allocation failure injected on the host) while the context keeps working."""
import numpy as np
import pytest

from multislice_gb300 import MslError, specimen as S
from multislice_gb300 import _abi
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _poisoned(torch, shape, dtype, pad=4096):
    """A device buffer of `shape` inside a NaN-filled allocation (pad guard elements each side)."""
    n = int(np.prod(shape))
    full = torch.full((n + 2 * pad,), float("nan"), dtype=dtype, device="cuda")
    return full, full[pad:pad + n].view(*shape)


def _guards_intact(torch, full, pad=4096):
    return bool(torch.isnan(full[:pad]).all()) and bool(torch.isnan(full[-pad:]).all())


def test_outputs_stay_inside_their_buffers(ctx):
    torch = pytest.importorskip("torch")
    spec = S.srtio3(2, 2, 2)
    n, nsl = 128, 4
    vf, v = _poisoned(torch, (nsl, n, n), torch.float32)
    ctx.potential(spec, n, n, nsl, 3.0, out=v)
    assert _guards_intact(torch, vf) and not torch.isnan(v).any()
    tf, t = _poisoned(torch, (nsl, n, n, 2), torch.float32)
    ctx.transmission(v, spec.ax, spec.by, 200.0, out=t)
    assert _guards_intact(torch, tf) and not torch.isnan(t).any()
    wf, w = _poisoned(torch, (3, n, n, 2), torch.float32)
    w[..., 0] = 1.0
    w[..., 1] = 0.0
    ctx.multislice(t, spec.cz / nsl, [0, 1, 2, 3] * 2, spec.ax, spec.by, 200.0, psi=w)
    assert _guards_intact(torch, wf) and not torch.isnan(w).any()
    xy = S.raster(0.0, spec.ax / 2, 0.0, spec.by / 2, 3, 3)
    df_, d = _poisoned(torch, (9, 2, 2), torch.float64)
    k_ap = float(S.mrad_to_k(20.0, 200.0))
    ctx.stem_scan(t, spec.cz / nsl, np.arange(8) % nsl, spec.ax, spec.by, 200.0, k_ap, xy,
                  [(0.0, k_ap), (2 * k_ap, 4 * k_ap)], checkpoints=[3, 7], out=d)
    assert _guards_intact(torch, df_) and not torch.isnan(d).any()
    ref = ctx.stem_scan(t.cpu().numpy().view(np.complex64)[..., 0], spec.cz / nsl, np.arange(8) % nsl,
                        spec.ax, spec.by, 200.0, k_ap, xy, [(0.0, k_ap), (2 * k_ap, 4 * k_ap)],
                        checkpoints=[3, 7])
    assert np.array_equal(d.cpu().numpy(), ref)


def test_memory_cap_fails_cleanly_and_batches_within_it():
    from multislice_gb300 import Context
    spec = S.srtio3(4, 4, 4)
    with Context(0) as c:
        n = 512
        v = c.potential(spec, n, n, 4, 1.9)
        t = c.transmission(v, spec.ax, spec.by, 200.0)
        xy = S.raster(0.0, spec.ax / 4, 0.0, spec.by / 4, 8, 8)
        k_ap = float(S.mrad_to_k(25.0, 200.0))
        det = [(float(S.mrad_to_k(80.0, 200.0)), float(S.mrad_to_k(200.0, 200.0)))]
        free = c.stem_scan(t, spec.cz / 4, np.arange(8) % 4, spec.ax, spec.by, 200.0, k_ap, xy, det)
    with Context(0) as c:
        cap = 48 << 20                       # 48 MiB: 12 waves of 512^2 per batch
        c.set_memory_limit(cap)
        d = c.stem_scan(t, spec.cz / 4, np.arange(8) % 4, spec.ax, spec.by, 200.0, k_ap, xy, det)
        assert np.array_equal(d, free)       # batching under the cap is invisible
        assert 0 < c.memory_in_use() <= cap
        with pytest.raises(MslError) as e:   # 32 waves of 2 MiB do not fit
            c.multislice(t, spec.cz / 4, [0, 1], spec.ax, spec.by, 200.0, batch=32)
        assert e.value.code == _abi.MSL_E_NOMEM
        assert c.memory_in_use() <= cap
        w = c.multislice(t, spec.cz / 4, [0, 1, 2, 3], spec.ax, spec.by, 200.0, batch=2)
        ref = O.rel_l2(w[0], w[1])
        assert ref == 0.0 and np.isfinite(w).all()
