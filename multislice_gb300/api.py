"""Python host mirror of the reference's multislice entry points over libmsl.so.

Each method is a thin wrapper over one C-ABI call of include/msl.h.  Arrays are
numpy arrays (host memory; the library copies them in and out) or CUDA tensors
of the context's device (anything with ``data_ptr()``; used in place).

Reference entry points mirrored here:
  * ModelPotential::calculatePotentialGrid   -> Context.potential
    (ImageSimulation/LMultiSlice/ModelPotential.cu:27-99)
  * mulslice transmission set-up             -> Context.transmission
    (ImageSimulation/multislice/mulslice.cpp:414-421, :515-522)
  * cfpix::fft / cfpix::ifft                  -> Context.fft2d (cfpix.cpp:115-167)
  * mulslice coherent loop / ModelSimulated   -> Context.multislice
    (mulslice.cpp:706-739; LMultiSlice/ModelSimulated.cu:52-119)
  * MSProjectReuse.StartCalculations STEM loop -> Context.stem_scan
    (Musli console 1.3 (STEM) 2/MSProjectReuse.cs:170-362)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _abi
from ._abi import Atoms, Detectors, Grid, Job, Lens, MslError, Optics, Probe

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def fparams_table():
    """Kirkland's FPARAMS coefficients (104 x 12, row Z), as shipped in the reference."""
    return np.load(os.path.join(_DATA, "fparams.npy"))


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(getattr(a, "device", None), "type", "cpu") == "cuda"


def _ptr(a, dtype):
    """c_void_p for a C-contiguous numpy array of `dtype` or a contiguous CUDA tensor."""
    if _is_device(a):
        if not a.is_contiguous():
            raise ValueError("device tensors must be contiguous")
        return ctypes.c_void_p(a.data_ptr())
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise ValueError(f"expected a C-contiguous numpy array of {np.dtype(dtype)}")
    return ctypes.c_void_p(a.ctypes.data)


def _cshape(a):
    """Shape of a complex array; a float CUDA tensor with a trailing dim of 2 counts as complex."""
    if _is_device(a) and not a.is_complex() and a.shape[-1] == 2:
        return tuple(a.shape[:-1])
    return tuple(a.shape)


def _as(a, dtype):
    if _is_device(a):
        return a
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One GPU, one stream: wraps msl_ctx."""

    def __init__(self, device=0):
        self._lib = _abi.load()
        h = ctypes.c_void_p()
        rc = self._lib.msl_ctx_create(int(device), ctypes.byref(h))
        if rc != _abi.MSL_OK:
            raise MslError(rc, f"msl_ctx_create(device={device}) failed")
        self._h = h
        self.device = device

    # -------------------------------------------------------------- plumbing
    def close(self):
        if getattr(self, "_h", None):
            self._lib.msl_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != _abi.MSL_OK:
            raise MslError(rc, self._lib.msl_last_error(self._h).decode())

    @property
    def launches(self):
        """Kernels launched by this context so far."""
        return int(self._lib.msl_kernel_launches(self._h))

    def profile(self, on=True):
        """Enable (and reset) per-kernel-kind event timing on the context's stream."""
        self._check(self._lib.msl_profile_enable(self._h, 1 if on else 0))

    def profile_read(self):
        """{kind: (launches, total ms)} for row, col, potential, other."""
        out = {}
        for k, name in enumerate(("row", "col", "potential", "other")):
            n = ctypes.c_int64()
            ms = ctypes.c_double()
            self._check(self._lib.msl_profile_read(self._h, k, ctypes.byref(n), ctypes.byref(ms)))
            out[name] = (int(n.value), float(ms.value))
        return out

    def set_probe_batch(self, batch):
        self._check(self._lib.msl_set_probe_batch(self._h, int(batch)))

    FAMILIES = ("fast", "tma", "register", "tensor-core")

    def autotune(self, side, batch, reps=3):
        """Time every pair of pass families at `side` and keep the fastest;
        returns (row_family, col_family, times [3, 3] ms per slice step)."""
        rf, cf = ctypes.c_int(), ctypes.c_int()
        ms = np.zeros(9, np.float64)
        self._check(self._lib.msl_autotune(self._h, int(side), int(batch), int(reps), ctypes.byref(rf),
                                           ctypes.byref(cf), ms.ctypes.data))
        return rf.value, cf.value, ms.reshape(3, 3)

    def set_schedule(self, side, row_family, col_family):
        self._check(self._lib.msl_set_schedule(self._h, int(side), int(row_family), int(col_family)))

    def get_schedule(self, side):
        rf, cf = ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.msl_get_schedule(self._h, int(side), ctypes.byref(rf), ctypes.byref(cf)))
        return rf.value, cf.value

    def set_autotune(self, on):
        self._check(self._lib.msl_set_autotune(self._h, 1 if on else 0))

    def set_memory_limit(self, nbytes):
        """Cap the device memory of the context's work buffers (0: no cap)."""
        self._check(self._lib.msl_set_memory_limit(self._h, int(nbytes)))

    def memory_in_use(self):
        n = ctypes.c_size_t(0)
        self._check(self._lib.msl_memory_in_use(self._h, ctypes.byref(n)))
        return n.value

    @staticmethod
    def _optics(kev, bandlimit=2.0 / 3.0, tilt=(0.0, 0.0), f32_prop_args=False):
        return Optics(float(kev), float(bandlimit), float(tilt[0]), float(tilt[1]),
                      1 if f32_prop_args else 0)

    # ------------------------------------------------------------- potential
    def potential(self, spec, nx, ny, nslice, radius, fparams=None, out=None):
        """Projected potential V_z (V*A) per slice, float32 [nslice, nx, ny]."""
        fp = np.ascontiguousarray(fparams_table() if fparams is None else fparams, np.float64)
        x = np.ascontiguousarray(spec.x, np.float64)
        y = np.ascontiguousarray(spec.y, np.float64)
        z = np.ascontiguousarray(spec.z, np.float64)
        Z = np.ascontiguousarray(spec.Z, np.int32)
        at = Atoms(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, Z.ctypes.data, float(spec.cz))
        g = Grid(int(nx), int(ny), float(spec.ax), float(spec.by))
        if out is None:
            out = np.empty((nslice, nx, ny), np.float32)
        self._check(self._lib.msl_potential_build(self._h, ctypes.byref(at), _ptr(fp, np.float64),
                                                  ctypes.byref(g), int(nslice), float(radius),
                                                  _ptr(out, np.float32)))
        return out

    # ---------------------------------------------------------- transmission
    def transmission(self, v, ax, by, kev, bandlimit=2.0 / 3.0, out=None):
        """Band-limited exp(i sigma V) per layer, complex64 [nlayer, nx, ny]."""
        v = _as(v, np.float32)
        nl, nx, ny = v.shape
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit)
        if out is None:
            out = np.empty((nl, nx, ny), np.complex64)
        self._check(self._lib.msl_transmission_build(self._h, ctypes.byref(g), ctypes.byref(o),
                                                     _ptr(v, np.float32), nl, _ptr(out, np.complex64)))
        return out

    # ------------------------------------------------------------------- fft
    def fft2d(self, psi, ax, by, direction):
        """In-place Kirkland fft (+1, exp(+i), unscaled) or ifft (-1, exp(-i), 1/(nx ny))."""
        shp = _cshape(psi)
        nx, ny = shp[-2], shp[-1]
        batch = int(np.prod(shp[:-2])) if len(shp) > 2 else 1
        g = Grid(nx, ny, float(ax), float(by))
        self._check(self._lib.msl_fft2d(self._h, ctypes.byref(g), _ptr(psi, np.complex64), batch,
                                        int(direction)))
        return psi

    # ------------------------------------------------------------ multislice
    def multislice(self, trans, dz, layer_seq, ax, by, kev, psi=None, batch=1,
                   bandlimit=2.0 / 3.0, tilt=(0.0, 0.0), f32_prop_args=False):
        """Exit waves of the coherent slice loop; psi=None starts from a plane wave."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit, tilt, f32_prop_args)
        plane = psi is None
        if plane:
            psi = np.empty((batch, nx, ny), np.complex64)
        else:
            shp = _cshape(psi)
            batch = int(np.prod(shp[:-2])) if len(shp) > 2 else 1
        self._check(self._lib.msl_multislice(self._h, ctypes.byref(g), ctypes.byref(o),
                                             _ptr(trans, np.complex64), nt, _ptr(dz, np.float64),
                                             _ptr(seq, np.int32), len(seq), _ptr(psi, np.complex64),
                                             batch, 1 if plane else 0))
        return psi

    # ------------------------------------------------------------ CTEM image
    @staticmethod
    def _lens(cs, df, k_obj, df_spread=0.0, df_step=0.0, astig=(0.0, 0.0, 0.0, 0.0)):
        return Lens(float(cs), float(df), float(k_obj), float(df_spread), float(df_step),
                    *[float(v) for v in astig])

    def ctem_image(self, trans, dz, layer_seq, ax, by, kev, cs, df, k_obj, psi=None, batch=1,
                   df_spread=0.0, df_step=0.0, weight=1.0, image=None, exit_intensity=None,
                   bandlimit=2.0 / 3.0, astig=(0.0, 0.0, 0.0, 0.0)):
        """Image intensity (FP64, accumulated into `image`) through an objective lens
        (mulslice.cpp:539-676); returns (image, exit waves, exit intensity)."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit)
        ln = self._lens(cs, df, k_obj, df_spread, df_step, astig)
        plane = psi is None
        if plane:
            psi = np.empty((batch, nx, ny), np.complex64)
        else:
            shp = _cshape(psi)
            batch = int(np.prod(shp[:-2])) if len(shp) > 2 else 1
        if image is None:
            image = np.zeros((nx, ny), np.float64)
        eptr = None if exit_intensity is None else _ptr(exit_intensity, np.float64)
        self._check(self._lib.msl_ctem_image(self._h, ctypes.byref(g), ctypes.byref(o),
                                             _ptr(trans, np.complex64), nt, _ptr(dz, np.float64),
                                             _ptr(seq, np.int32), len(seq), ctypes.byref(ln),
                                             _ptr(psi, np.complex64), batch, 1 if plane else 0,
                                             float(weight), _ptr(image, np.float64), eptr))
        return image, psi, exit_intensity

    def partial_coherence(self, trans, dz, layer_seq, ax, by, kev, cs, df, k_obj, acmin, acmax,
                          df_spread=0.0, df_step=0.0, astig=(0.0, 0.0, 0.0, 0.0),
                          bandlimit=2.0 / 3.0):
        """Kirkland's partial-coherence image (illumination angles acmin..acmax in rad);
        returns (image float64 [nx, ny], number of angles)."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit)
        ln = self._lens(cs, df, k_obj, df_spread, df_step, astig)
        img = np.empty((nx, ny), np.float64)
        na = ctypes.c_int()
        self._check(self._lib.msl_ctem_partial_coherence(
            self._h, ctypes.byref(g), ctypes.byref(o), _ptr(trans, np.complex64), nt,
            _ptr(dz, np.float64), _ptr(seq, np.int32), len(seq), ctypes.byref(ln), float(acmin),
            float(acmax), _ptr(img, np.float64), ctypes.byref(na)))
        return img, int(na.value)

    def frozen_phonon(self, spec, nx, ny, nslice, radius, kev, cs, df, k_obj, nconfig, sigma, seed,
                      df_spread=0.0, df_step=0.0, fparams=None, bandlimit=2.0 / 3.0,
                      want_exit=True):
        """Configuration-averaged image and exit-wave intensity, float64 [nx, ny] each."""
        fp = np.ascontiguousarray(fparams_table() if fparams is None else fparams, np.float64)
        x = np.ascontiguousarray(spec.x, np.float64)
        y = np.ascontiguousarray(spec.y, np.float64)
        z = np.ascontiguousarray(spec.z, np.float64)
        Z = np.ascontiguousarray(spec.Z, np.int32)
        at = Atoms(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, Z.ctypes.data, float(spec.cz))
        g = Grid(int(nx), int(ny), float(spec.ax), float(spec.by))
        o = self._optics(kev, bandlimit)
        ln = self._lens(cs, df, k_obj, df_spread, df_step)
        img = np.empty((nx, ny), np.float64)
        ex = np.empty((nx, ny), np.float64) if want_exit else None
        self._check(self._lib.msl_frozen_phonon(self._h, ctypes.byref(at), _ptr(fp, np.float64),
                                                ctypes.byref(g), int(nslice), float(radius),
                                                ctypes.byref(o), ctypes.byref(ln), int(nconfig),
                                                float(sigma), int(seed), _ptr(img, np.float64),
                                                None if ex is None else _ptr(ex, np.float64)))
        return img, ex

    def stem_scan_phonon(self, spec, nx, ny, nslice, radius, kev, k_ap, probe_xy, det_k,
                         nconfig, sigma, seed, checkpoints=None, df=0.0, cs=0.0, k_ap_in=0.0,
                         fparams=None, bandlimit=2.0 / 3.0, out=None):
        """Frozen-phonon STEM: detector sums added over nconfig configurations,
        float64 [nprobe, ncheck, ndet] (msl_stem_scan_phonon)."""
        fp = np.ascontiguousarray(fparams_table() if fparams is None else fparams, np.float64)
        x = np.ascontiguousarray(spec.x, np.float64)
        y = np.ascontiguousarray(spec.y, np.float64)
        z = np.ascontiguousarray(spec.z, np.float64)
        Z = np.ascontiguousarray(spec.Z, np.int32)
        at = Atoms(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, Z.ctypes.data, float(spec.cz))
        g = Grid(int(nx), int(ny), float(spec.ax), float(spec.by))
        o = self._optics(kev, bandlimit)
        if checkpoints is None:
            checkpoints = [nslice - 1]
        cps = np.ascontiguousarray(checkpoints, np.int32)
        xy = np.ascontiguousarray(probe_xy, np.float64).reshape(-1, 2)
        det = np.asarray(det_k, np.float64).reshape(-1, 2)
        kin = np.ascontiguousarray(det[:, 0])
        kout = np.ascontiguousarray(det[:, 1])
        dets = Detectors(len(det), kin.ctypes.data, kout.ctypes.data)
        pr = Probe(float(k_ap_in), float(k_ap), float(df), float(cs))
        if out is None:
            out = np.empty((len(xy), len(cps), len(det)), np.float64)
        self._check(self._lib.msl_stem_scan_phonon(self._h, ctypes.byref(at), _ptr(fp, np.float64),
                                                   ctypes.byref(g), int(nslice), float(radius),
                                                   ctypes.byref(o), ctypes.byref(pr), _ptr(xy, np.float64),
                                                   len(xy), ctypes.byref(dets), _ptr(cps, np.int32),
                                                   len(cps), int(nconfig), float(sigma), int(seed),
                                                   _ptr(out, np.float64)))
        return out

    # ---------------------------------------------------------- uneven jobs
    def run_jobs(self, jobs, bandlimit=2.0 / 3.0):
        """Run many independent slice loops at once (msl_run_jobs).

        jobs: list of dicts with trans [ntrans, nx, ny] complex64, ax, by, kev, dz, layer_seq
        and optionally probe=(k_ap, x, y[, df, cs]).  Returns the exit waves."""
        keep = []
        arr = (Job * len(jobs))()
        outs = []
        for j, d in enumerate(jobs):
            t = _as(d["trans"], np.complex64)
            nt, nx, ny = _cshape(t)
            dz = np.ascontiguousarray(np.broadcast_to(np.asarray(d["dz"], np.float64), (nt,)))
            seq = np.ascontiguousarray(d["layer_seq"], np.int32)
            out = d.get("out")
            if out is None:
                out = np.empty((nx, ny), np.complex64)
            keep += [t, dz, seq]
            outs.append(out)
            jb = arr[j]
            jb.grid = Grid(nx, ny, float(d["ax"]), float(d["by"]))
            jb.kev = float(d["kev"])
            jb.trans = _ptr(t, np.complex64).value
            jb.ntrans = nt
            jb.dz = dz.ctypes.data
            jb.layer_seq = seq.ctypes.data
            jb.nslice = len(seq)
            pr = d.get("probe")
            if pr is None:
                jb.illumination = _abi.PLANE_WAVE
            else:
                k_ap, x, y = pr[:3]
                df = pr[3] if len(pr) > 3 else 0.0
                cs = pr[4] if len(pr) > 4 else 0.0
                jb.illumination = _abi.PROBE
                jb.probe = Probe(0.0, float(k_ap), float(df), float(cs))
                jb.probe_x, jb.probe_y = float(x), float(y)
            jb.exit_wave = _ptr(out, np.complex64).value
        self._check(self._lib.msl_run_jobs(self._h, ctypes.byref(arr), len(jobs), float(bandlimit)))
        return outs

    # ------------------------------------------------------------------ STEM
    def stem_scan(self, trans, dz, layer_seq, ax, by, kev, k_ap, probe_xy, det_k,
                  checkpoints=None, df=0.0, cs=0.0, k_ap_in=0.0, bandlimit=2.0 / 3.0,
                  f32_prop_args=False, out=None, resident=False):
        """Annular detector sums, float64 [nprobe, ncheck, ndet] (reference scale).
        resident=True runs the on-chip slice loop (msl_stem_scan_resident, 256^2)."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        if checkpoints is None:
            checkpoints = [len(seq) - 1]
        cps = np.ascontiguousarray(checkpoints, np.int32)
        xy = np.ascontiguousarray(probe_xy, np.float64).reshape(-1, 2)
        det = np.asarray(det_k, np.float64).reshape(-1, 2)
        kin = np.ascontiguousarray(det[:, 0])
        kout = np.ascontiguousarray(det[:, 1])
        dets = Detectors(len(det), kin.ctypes.data, kout.ctypes.data)
        pr = Probe(float(k_ap_in), float(k_ap), float(df), float(cs))
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit, (0.0, 0.0), f32_prop_args)
        if out is None:
            out = np.empty((len(xy), len(cps), len(det)), np.float64)
        fn = self._lib.msl_stem_scan_resident if resident else self._lib.msl_stem_scan
        self._check(fn(self._h, ctypes.byref(g), ctypes.byref(o),
                                            _ptr(trans, np.complex64), nt, _ptr(dz, np.float64),
                                            _ptr(seq, np.int32), len(seq), ctypes.byref(pr),
                                            _ptr(xy, np.float64), len(xy), ctypes.byref(dets),
                                            _ptr(cps, np.int32), len(cps), _ptr(out, np.float64)))
        return out


    def stem_exit_waves(self, trans, dz, layer_seq, ax, by, kev, k_ap, probe_xy, df=0.0, cs=0.0, k_ap_in=0.0,
                        bandlimit=2.0 / 3.0, out=None):
        """Real-space exit waves of the scan's probes, complex64 [nprobe, nx, ny]
        (or into `out`, e.g. a torch device tensor [nprobe, nx, ny, 2])."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        xy = np.ascontiguousarray(probe_xy, np.float64).reshape(-1, 2)
        pr = Probe(float(k_ap_in), float(k_ap), float(df), float(cs))
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit)
        if out is None:
            out = np.empty((len(xy), nx, ny), np.complex64)
        self._check(self._lib.msl_stem_exit_waves(self._h, ctypes.byref(g), ctypes.byref(o),
                                                  _ptr(trans, np.complex64), nt, _ptr(dz, np.float64),
                                                  _ptr(seq, np.int32), len(seq), ctypes.byref(pr),
                                                  _ptr(xy, np.float64), len(xy), _ptr(out, np.complex64)))
        return out

    def stem_scan_closure(self, net, trans, dz, layer_seq, ax, by, kev, k_ap, probe_xy, det_k, df=0.0, cs=0.0,
                          k_ap_in=0.0, bandlimit=2.0 / 3.0, out=None):
        """Detector sums [nprobe, ndet] of coarse-slice exit waves corrected by the closure."""
        trans = _as(trans, np.complex64)
        nt, nx, ny = _cshape(trans)
        dz = np.ascontiguousarray(np.broadcast_to(np.asarray(dz, np.float64), (nt,)))
        seq = np.ascontiguousarray(layer_seq, np.int32)
        xy = np.ascontiguousarray(probe_xy, np.float64).reshape(-1, 2)
        det = np.asarray(det_k, np.float64).reshape(-1, 2)
        kin = np.ascontiguousarray(det[:, 0])
        kout = np.ascontiguousarray(det[:, 1])
        dets = Detectors(len(det), kin.ctypes.data, kout.ctypes.data)
        pr = Probe(float(k_ap_in), float(k_ap), float(df), float(cs))
        g = Grid(nx, ny, float(ax), float(by))
        o = self._optics(kev, bandlimit)
        if out is None:
            out = np.empty((len(xy), len(det)), np.float64)
        self._check(self._lib.msl_stem_scan_closure(self._h, net._h, ctypes.byref(g), ctypes.byref(o),
                                                    _ptr(trans, np.complex64), nt, _ptr(dz, np.float64),
                                                    _ptr(seq, np.int32), len(seq), ctypes.byref(pr),
                                                    _ptr(xy, np.float64), len(xy), ctypes.byref(dets),
                                                    _ptr(out, np.float64)))
        return out


def phonon_displacements(seed, config, natom, sigma):
    """Frozen-phonon displacements [natom, 3] of configuration `config` (msl_phonon_displacements)."""
    d = np.empty((natom, 3), np.float64)
    rc = _abi.load().msl_phonon_displacements(int(seed), int(config), int(natom), float(sigma),
                                               ctypes.c_void_p(d.ctypes.data))
    if rc != _abi.MSL_OK:
        raise MslError(rc, "msl_phonon_displacements failed")
    return d


def wavelength(kev):
    return _abi.load().msl_wavelength(float(kev))


def sigma(kev):
    return _abi.load().msl_sigma(float(kev))


class Closure:
    """The learned coarse-slice closure (msl_closure_*): a complex 3x3
    convolutional network correcting a coarse-slice exit wave toward the
    fine-slice one.  Waves are complex64 [batch, h, w] (numpy, or torch device
    tensors of shape [batch, h, w, 2] float32)."""

    def __init__(self, ctx, seed=0):
        self.ctx = ctx
        self._lib = ctx._lib
        h = ctypes.c_void_p()
        ctx._check(self._lib.msl_closure_create(ctx._h, int(seed), ctypes.byref(h)))
        self._h = h

    @staticmethod
    def param_count():
        return int(_abi.load().msl_closure_param_count())

    def close(self):
        if self._h:
            self._lib.msl_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        p = np.empty(self.param_count(), np.float32)
        self.ctx._check(self._lib.msl_closure_get_params(self.ctx._h, self._h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.param_count()
        self.ctx._check(self._lib.msl_closure_set_params(self.ctx._h, self._h, p.ctypes.data))

    @staticmethod
    def _wave_ptr(w):
        if hasattr(w, "data_ptr"):
            return ctypes.c_void_p(w.data_ptr()), tuple(w.shape[:3])
        assert w.dtype == np.complex64 and w.flags.c_contiguous
        return ctypes.c_void_p(w.ctypes.data), w.shape

    def apply(self, psi):
        """psi <- psi + s net(psi / s), in place; returns psi."""
        if not hasattr(psi, "data_ptr"):
            psi = np.ascontiguousarray(psi, np.complex64)
        ptr, (b, h, w) = self._wave_ptr(psi)
        self.ctx._check(self._lib.msl_closure_apply(self.ctx._h, self._h, ptr, b, h, w))
        return psi

    def gradients(self, coarse, fine):
        pc, (b, h, w) = self._wave_ptr(coarse)
        pf, _ = self._wave_ptr(fine)
        g = np.empty(self.param_count(), np.float32)
        loss = ctypes.c_double()
        self.ctx._check(self._lib.msl_closure_gradients(self.ctx._h, self._h, pc, pf, b, h, w,
                                                        g.ctypes.data, ctypes.byref(loss)))
        return loss.value, g

    def train_step(self, coarse, fine, lr):
        pc, (b, h, w) = self._wave_ptr(coarse)
        pf, _ = self._wave_ptr(fine)
        loss = ctypes.c_double()
        self.ctx._check(self._lib.msl_closure_train_step(self.ctx._h, self._h, pc, pf, b, h, w, float(lr),
                                                         ctypes.byref(loss)))
        return loss.value
