"""msl_multislice replays small slice loops as a cached CUDA graph: a call seen
twice in a row is captured, then replayed while it repeats.  Every call --
direct, capturing, replaying, after a key change -- gives the same exit wave
bit for bit as a fresh context's first (direct) call."""
import numpy as np
import pytest

from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _layers(seed, nt=3, n=128):
    rng = np.random.default_rng(seed)
    V = np.zeros((nt, n, n))
    for l in range(nt):
        ix, iy = rng.integers(0, n, 12), rng.integers(0, n, 12)
        V[l, ix, iy] = rng.uniform(50, 400, 12)
    return O.transmission(V, 200.0, 14.0, 14.0, np.complex64)


def test_repeated_calls_replay_the_graph_bit_for_bit():
    from multislice_gb300 import Context
    t = _layers(3)
    seq_a = np.array([0, 1, 2, 1, 0, 2, 2, 1])
    seq_b = np.array([2, 2, 1, 0, 1, 0, 0, 1, 2, 1])
    with Context(0) as fresh:
        ref_a = fresh.multislice(t, 1.5, seq_a, 14.0, 14.0, 200.0)
    with Context(0) as fresh:
        ref_b = fresh.multislice(t, 1.5, seq_b, 14.0, 14.0, 200.0)
    with Context(0) as c:
        n0 = c.launches
        outs = [c.multislice(t, 1.5, seq_a, 14.0, 14.0, 200.0) for _ in range(4)]   # direct, capture, replay x2
        per_call = (c.launches - n0) / 4
        assert per_call == 2 * len(seq_a) + 1     # replays count their launches too
        for w in outs:
            assert np.array_equal(w, ref_a)
        for _ in range(3):                                                          # key change, back again
            assert np.array_equal(c.multislice(t, 1.5, seq_b, 14.0, 14.0, 200.0), ref_b)
            assert np.array_equal(c.multislice(t, 1.5, seq_a, 14.0, 14.0, 200.0), ref_a)
        assert np.array_equal(c.multislice(t, 1.5, seq_a, 14.0, 14.0, 200.0), ref_a)
        props = [O.propagator_tables(128, 128, 14.0, 14.0, 200.0, 1.5, precision="f64")] * 3
        wo, _ = O.multislice(np.ones((128, 128), np.complex128), t.astype(np.complex128), props, seq_a,
                             O.band_mask(128, 128, 14.0, 14.0))
        assert O.rel_l2(outs[-1][0], wo) < 2e-5


def test_new_thickness_updates_the_tables_under_a_replayed_graph():
    """The propagator tables are uploaded on every call: a replayed graph sees
    the current call's slice thickness."""
    from multislice_gb300 import Context
    t = _layers(5)
    seq = np.array([0, 1, 2, 0, 1, 2])
    with Context(0) as c:
        for _ in range(3):
            c.multislice(t, 1.5, seq, 14.0, 14.0, 200.0)
        w = c.multislice(t, 2.25, seq, 14.0, 14.0, 200.0)
    with Context(0) as fresh:
        ref = fresh.multislice(t, 2.25, seq, 14.0, 14.0, 200.0)
    assert np.array_equal(w, ref)
