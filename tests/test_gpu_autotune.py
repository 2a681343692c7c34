"""The pass-schedule autotuner: every pair of kernel families computes the same
slice loop (against the oracle), the tuner keeps the pair it measured fastest,
and automatic tuning on first use leaves results within the same bounds."""
import numpy as np
import pytest

from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [256, 384, 512])
def test_every_schedule_matches_oracle(ctx, n):
    rng = np.random.default_rng(n)
    t = np.exp(1j * 0.3 * rng.standard_normal((2, n, n))).astype(np.complex64)
    psi = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64)
    ax = by = 0.1 * n
    seq = [0, 1, 0]
    mask = O.band_mask(n, n, ax, by)
    props = [O.propagator_tables(n, n, ax, by, 200.0, 1.5, precision="f64")] * 2
    ref, _ = O.multislice(psi.astype(np.complex128), t.astype(np.complex128), props, seq, mask)
    try:
        for rf in range(3):
            for cf in range(3):
                ctx.set_schedule(n, rf, cf)
                assert ctx.get_schedule(n) == (rf, cf)
                got = ctx.multislice(t, 1.5, seq, ax, by, 200.0, psi=psi.copy())
                assert O.rel_l2(got, ref) < 2e-5, (rf, cf)
    finally:
        ctx.set_schedule(n, 0, 0)


def test_autotune_keeps_the_fastest_pair(ctx):
    rf, cf, ms = ctx.autotune(512, 64, reps=2)
    assert np.all(ms > 0)
    assert ms[rf, cf] == ms.min()
    assert ctx.get_schedule(512) == (rf, cf)
    ctx.set_schedule(512, 0, 0)


def test_automatic_tuning_on_first_use():
    from multislice_gb300 import Context
    rng = np.random.default_rng(1)
    n = 768
    t = np.exp(1j * 0.2 * rng.standard_normal((1, n, n))).astype(np.complex64)
    with Context(0) as c:
        c.set_autotune(True)
        got = c.multislice(t, 1.0, [0, 0], 60.0, 60.0, 200.0)
        sched = c.get_schedule(n)
        c.set_schedule(n, 0, 0)
        ref = c.multislice(t, 1.0, [0, 0], 60.0, 60.0, 200.0)
    assert all(0 <= f < 3 for f in sched)
    assert O.rel_l2(got, ref) < 2e-5
