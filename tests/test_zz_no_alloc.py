"""msl_multislice_noalloc against msl_multislice, through the C ABI.

Some callers cannot allocate GPU memory: code embedded in an application whose
own pool allocator owns the device's memory, or a latency-critical loop where a
cudaMalloc/cudaFree would stall the device.  They hand the library their own
device buffers and call msl_multislice_noalloc, which keeps its small tables in
a fixed device array instead of allocating.  This file checks that such a call
gives the same exit waves as the allocating entry point, on two calls in a row
with different inputs (the shared array must not carry anything over), and that
requests beyond the array's limits are refused.  It is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from multislice_gb300 import _abi
from multislice_gb300._abi import Grid, Optics
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu


def _noalloc(lib, trans_dev, dz, seq, ax, by, kev, psi_dev, batch, plane_wave,
             bandlimit=2.0 / 3.0, f32_prop_args=0):
    nt, nx, ny = trans_dev.shape[:3]
    g = Grid(nx, ny, float(ax), float(by))
    o = Optics(float(kev), float(bandlimit), 0.0, 0.0, int(f32_prop_args))
    dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
    seq = np.ascontiguousarray(seq, np.int32)
    return lib.msl_multislice_noalloc(ctypes.byref(g), ctypes.byref(o),
                                      ctypes.c_void_p(trans_dev.data_ptr()), nt,
                                      ctypes.c_void_p(dz.ctypes.data), ctypes.c_void_p(seq.ctypes.data),
                                      len(seq), ctypes.c_void_p(psi_dev.data_ptr()), batch,
                                      plane_wave, None)


def _to_dev(torch, a):
    a = np.ascontiguousarray(a, np.complex64)
    return torch.from_numpy(a.view(np.float32).reshape(a.shape + (2,))).cuda()


def _to_host(t):
    f = t.cpu().numpy()
    return (f[..., 0] + 1j * f[..., 1]).astype(np.complex64)


def test_noalloc_matches_allocating_entry_point_twice(golden):
    import torch

    from multislice_gb300 import Context

    lib = _abi.load()
    torch.cuda.set_device(0)
    with Context(0) as ctx:
        # call 1: the Si 64^2 golden case, plane-wave start, 32 slices over 8 layers
        G = golden("si_small.npz")
        ax, by, dz = float(G["ax"]), float(G["by"]), float(G["dz"])
        t1 = _to_dev(torch, G["t"])
        psi1 = torch.empty((1, 64, 64, 2), dtype=torch.float32, device="cuda")
        rc = _noalloc(lib, t1, dz, G["seq"], ax, by, 200.0, psi1, 1, 1)
        assert rc == _abi.MSL_OK
        ref1 = ctx.multislice(G["t"], dz, G["seq"], ax, by, 200.0)
        got1 = _to_host(psi1)
        assert O.rel_l2(got1, ref1) < 1e-6
        assert O.rel_l2(got1[0], G["wave"]) < 1e-5

        # call 2: another grid, three layers of different thickness, a batch of
        # entrance waves, float propagator arguments and a narrower band limit
        rng = np.random.default_rng(4)
        n = 128
        t = np.exp(1j * 0.3 * rng.standard_normal((3, n, n))).astype(np.complex64)
        psi = (rng.standard_normal((3, n, n)) + 1j * rng.standard_normal((3, n, n))).astype(np.complex64)
        dzs = [1.5, 2.0, 0.75]
        seq = [0, 1, 2, 1, 0, 2, 2]
        t2 = _to_dev(torch, t)
        psi2 = _to_dev(torch, psi)
        rc = _noalloc(lib, t2, dzs, seq, 17.0, 19.0, 300.0, psi2, 3, 0, bandlimit=0.5, f32_prop_args=1)
        assert rc == _abi.MSL_OK
        ref2 = ctx.multislice(t, dzs, seq, 17.0, 19.0, 300.0, psi=psi.copy(), bandlimit=0.5,
                              f32_prop_args=True)
        assert O.rel_l2(_to_host(psi2), ref2) < 1e-6


@pytest.mark.parametrize("n", [1024, 2048])
def test_noalloc_large_sides_twice(n):
    """1024 carries the two-stage row kernel's appended twiddle table and 2048
    fills the array's twiddle slot exactly; two calls in a row, different inputs."""
    import torch

    from multislice_gb300 import Context

    lib = _abi.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(n)
    with Context(0) as ctx:
        for call in range(2):
            nt = 2 + call
            t = np.exp(1j * 0.2 * rng.standard_normal((nt, n, n))).astype(np.complex64)
            psi = (rng.standard_normal((1, n, n)) + 1j * rng.standard_normal((1, n, n))).astype(np.complex64)
            dzs = [1.0 + 0.5 * l for l in range(nt)]
            seq = list(range(nt)) + [0]
            ax = 0.1 * n + call
            t_d = _to_dev(torch, t)
            psi_d = _to_dev(torch, psi)
            rc = _noalloc(lib, t_d, dzs, seq, ax, ax + 1.0, 200.0, psi_d, 1, 0)
            assert rc == _abi.MSL_OK
            ref = ctx.multislice(t, dzs, seq, ax, ax + 1.0, 200.0, psi=psi.copy())
            assert O.rel_l2(_to_host(psi_d), ref) < 1e-6
            del t_d, psi_d


def test_noalloc_refuses_requests_beyond_its_limits():
    import torch

    lib = _abi.load()
    torch.cuda.set_device(0)
    t = torch.zeros((65, 64, 64, 2), dtype=torch.float32, device="cuda")
    psi = torch.zeros((1, 64, 64, 2), dtype=torch.float32, device="cuda")
    # more layers than the fixed array holds
    assert _noalloc(lib, t, 1.0, [0], 10.0, 10.0, 200.0, psi, 1, 1) == _abi.MSL_E_ARG
    # host buffers are refused: the caller owns device memory
    host = np.zeros((1, 64, 64), np.complex64)
    g = Grid(64, 64, 10.0, 10.0)
    o = Optics(200.0, 2.0 / 3.0, 0.0, 0.0, 0)
    dz = np.ones(1)
    seq = np.zeros(1, np.int32)
    rc = lib.msl_multislice_noalloc(ctypes.byref(g), ctypes.byref(o), ctypes.c_void_p(t.data_ptr()),
                                    1, ctypes.c_void_p(dz.ctypes.data), ctypes.c_void_p(seq.ctypes.data),
                                    1, ctypes.c_void_p(host.ctypes.data), 1, 1, None)
    assert rc == _abi.MSL_E_ARG
