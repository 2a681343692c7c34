"""Job-file front ends: run the reference's own XML job files on the GPU.

Two formats exist in the reference:

* LMultiSlice's `<action>` job (ImageSimulation/LMultiSlice/Dispatcher.cu:25-159):
  io/fileNameInput (.coo), io/fileNameOutput, image/nx, ny, dpa, slicing/radiuc,
  numberslices, microscope/aperture (mrad), cs (mm), defocus (nm), keV.  Runs a
  CTEM plane-wave multislice and an objective-lens image and writes MRC files
  (Dispatcher.cu:209-223): <out>_pt.mrc (potential), <out>_wave.mrc (exit wave)
  and <out>.mrc (image intensity).
* The C# STEM driver's `<Calculation_parameters>` job (Musli console 1.3 (STEM) 2/
  MSProjectInfo.cs:10-72; sample Musli/new/test.xml): ModelFileName, NSlices
  (slices per unit cell), atrad, N, M, E (V), IniWaveType (PlaneWave, Converged,
  STEMshift), BeamShift, ConvAngles and DetectorAngles (1/A, outer then inner),
  Df, Cs (A), ThWaves (thickness checkpoints, A).  The unit cell is repeated
  along the beam until the last checkpoint (MSReuseCalculator.cs:36-92).
  IniWaveType Precalculated resumes from a saved .wav (IniWaveFileName): its
  trailer must match the cell (a, b, gamma within 1e-5) and the grid, and sets
  the energy and the start thickness; the checkpoints stay absolute
  (MSProject.cs:423-440, MSProjectReuse.cs:337).
  Results are written in the driver's own formats (csfiles.py) and as MRC:
  .wav exit waves (IsSaveWaves, default on), .cbed diffraction patterns
  (IsSaveDiffractions), .stem images, and the slices' phase gratings as .slice
  files under "Slice stack" (SaveSlices, MSProjectReuse.cs:443, :527-560).

What differs from the reference, by design: the potential is always Kirkland's
FPARAMS form (the C# PotType families are not rebuilt here); the cutoff radius
is capped below half the cell (single minimum image); LMultiSlice's `aperture`
is applied as a hard objective aperture (its own Es envelope squares k twice,
ModelSimulated.cu / kernel.cu:86-92).
"""
from __future__ import annotations

import math
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import specimen as S
from .api import Context, wavelength
from .csfiles import read_wav, write_cbed, write_slice, write_stem, write_wav
from .mrc import write_mrc


def _f(node, path, default=None, cast=float):
    el = node.find(path)
    if el is None or el.text is None or not el.text.strip():
        if default is None:
            raise ValueError(f"job file: <{path}> is required")
        return default
    return cast(el.text.strip().replace(",", "."))


def _bool(node, path, default):
    el = node.find(path)
    if el is None or el.text is None or not el.text.strip():
        return default
    return el.text.strip().lower() in ("true", "1")


def _doubles(node, path):
    el = node.find(path)
    if el is None:
        return []
    return [float(d.text) for d in el.iter("double")]


def _pairs(node, path):
    el = node.find(path)
    if el is None:
        return []
    return [[float(d.text) for d in arr.iter("double")] for arr in el.findall("ArrayOfDouble")]


def _resolve(base, name):
    return name if os.path.isabs(name) else os.path.join(base, name)


def _radius(r, spec):
    return min(float(r), 0.499 * min(spec.ax, spec.by))


def run_lmultislice(root, base_dir, ctx):
    """LMultiSlice <action>: potential -> CTEM exit wave -> objective-lens image, as MRC."""
    spec = S.read_coo(_resolve(base_dir, _f(root, "io/fileNameInput", cast=str)))
    out = _resolve(base_dir, _f(root, "io/fileNameOutput", cast=str))
    nx = int(_f(root, "image/nx"))
    ny = int(_f(root, "image/ny"))
    nslice = int(_f(root, "slicing/numberslices"))
    radius = _radius(_f(root, "slicing/radiuc"), spec)
    kev = _f(root, "microscope/keV")
    cs = _f(root, "microscope/cs") * 1.0e7          # mm -> A
    df = _f(root, "microscope/defocus") * 10.0      # nm -> A
    ap = _f(root, "microscope/aperture", 0.0)       # mrad
    k_obj = ap * 1e-3 / wavelength(kev) if ap > 0 else 1.0e3
    v = ctx.potential(spec, nx, ny, nslice, radius)
    t = ctx.transmission(v, spec.ax, spec.by, kev)
    img, psi, _ = ctx.ctem_image(t, spec.cz / nslice, np.arange(nslice), spec.ax, spec.by, kev, cs, df,
                                 k_obj)
    cell = (spec.ax, spec.by, spec.cz)
    write_mrc(out + "_pt.mrc", v, cell, ["projected potential V_z (V*A) per slice"])
    write_mrc(out + "_wave.mrc", psi[0], cell, ["exit wave"])
    write_mrc(out + ".mrc", img.astype(np.float32), cell, ["image intensity"])
    return {"potential": out + "_pt.mrc", "wave": out + "_wave.mrc", "image": out + ".mrc",
            "radius": radius}


def _slices_to(thicknesses, dz, nslice_cell):
    """Slice sequence over repeated cells up to the last thickness, and the
    checkpoint slice (0-based) of every thickness (first slice whose bottom
    reaches it, MSReuseCalculator.cs:58-78)."""
    cps = []
    total = 0.0
    s = 0
    target = sorted(thicknesses)
    for th in target:
        while total < th - 1e-9:
            total += dz
            s += 1
        cps.append(max(s - 1, 0))
    seq = np.arange(max(s, 1)) % nslice_cell
    return seq, cps


def run_musli(root, base_dir, ctx):
    """C# <Calculation_parameters>: PlaneWave / Converged exit waves or a STEMshift scan."""
    spec = S.read_coo(_resolve(base_dir, _f(root, "ModelFileName", cast=str)))
    stem = os.path.splitext(_resolve(base_dir, _f(root, "ModelFileName", cast=str)))[0]
    nsl = int(_f(root, "NSlices", 1))
    radius = _radius(_f(root, "atrad", 3.0), spec)
    nx = int(_f(root, "N", 512))
    ny = int(_f(root, "M", 512))
    E = _doubles(root, "E") or [100000.0]
    kev = E[0] / 1000.0
    ths = _doubles(root, "ThWaves") or [spec.cz]
    kind = _f(root, "IniWaveType", "PlaneWave", cast=str)
    start_wave, start_th = None, 0.0
    if kind == "Precalculated":
        start_wave, meta = read_wav(_resolve(base_dir, _f(root, "IniWaveFileName", cast=str)))
        if (abs(meta["a"] - spec.ax) > 1e-5 or abs(meta["b"] - spec.by) > 1e-5
                or abs(meta["gamma"] - math.pi / 2) > 1e-5 or (meta["n"], meta["m"]) != (nx, ny)):
            raise ValueError("parameters of the preloaded initial wave do not fit those of the model")
        kev = meta["kev"]
        start_th = meta["f9"]
    df = (_doubles(root, "Df") or [0.0])[0]
    cs = (_doubles(root, "Cs") or [0.0])[0]
    dz = spec.cz / nsl
    v = ctx.potential(spec, nx, ny, nsl, radius)
    t = ctx.transmission(v, spec.ax, spec.by, kev)
    seq, cps = _slices_to([max(th - start_th, 0.0) for th in ths], dz, nsl)
    results = {"checkpoints": cps, "thickness": ths}
    if _bool(root, "SaveSlices", False):
        sdir = os.path.join(os.path.dirname(stem), "Slice stack")
        os.makedirs(sdir, exist_ok=True)
        for i in range(nsl):
            write_slice(os.path.join(sdir, f"Slice_{i:04d}.slice"), t[i], spec.ax, spec.by, dz, i, nsl)
        results["slices"] = sdir
    if kind == "STEMshift":
        bs = _pairs(root, "BeamShift")
        (npx, npy), (x0, y0), (x1, y1) = bs[0], bs[1], bs[2]
        xy = S.raster(x0 * spec.ax, x1 * spec.ax, y0 * spec.by, y1 * spec.by, int(npx), int(npy))
        conv = _pairs(root, "ConvAngles")[0]
        dets = [(d[1] if len(d) > 1 else 0.0, d[0]) for d in _pairs(root, "DetectorAngles")]
        d = ctx.stem_scan(t, dz, seq, spec.ax, spec.by, kev, conv[0], xy, dets, checkpoints=cps,
                          df=df, cs=cs, k_ap_in=conv[1] if len(conv) > 1 else 0.0)
        img = d.reshape(int(npx), int(npy), len(cps), len(dets))
        for ic, th in enumerate(ths):
            for k in range(len(dets)):
                path = f"{stem}_stem_{th:g}A_det{k}"
                write_mrc(path + ".mrc", img[:, :, ic, k].astype(np.float32), (spec.ax, spec.by, th),
                          [f"STEM detector {k}, thickness {th:g} A"])
                write_stem(path + ".stem", img[:, :, ic, k], (x1 - x0, y1 - y0), th, kev)
        results["stem"] = img
        return results
    waves = []
    save_waves = _bool(root, "IsSaveWaves", True)
    save_diff = _bool(root, "IsSaveDiffractions", False)
    for ic, th in enumerate(ths):
        n = cps[ic] + 1
        if start_wave is not None:
            if th <= start_th + 1e-9:          # already reached: the loaded wave itself
                w = start_wave.astype(np.complex64)
            else:
                psi = np.ascontiguousarray(start_wave.astype(np.complex64)[None])
                w = ctx.multislice(t, dz, seq[:n], spec.ax, spec.by, kev, psi=psi)[0]
        elif kind == "Converged":
            conv = _pairs(root, "ConvAngles")[0]
            x, y = _pairs(root, "BeamShift")[0]
            job = dict(trans=t, ax=spec.ax, by=spec.by, kev=kev, dz=dz, layer_seq=seq[:n],
                       probe=(conv[0], x * spec.ax, y * spec.by, df, cs))
            w = ctx.run_jobs([job])[0]
        else:
            w = ctx.multislice(t, dz, seq[:n], spec.ax, spec.by, kev)[0]
        path = f"{stem}_wave_{th:g}A"
        write_mrc(path + ".mrc", w, (spec.ax, spec.by, th), [f"exit wave at {th:g} A"])
        if save_waves:
            write_wav(path + ".wav", w, spec.ax, spec.by, th, kev)
        if save_diff:
            # the spectrum after the checkpoint slice's propagator = forward transform of the exit wave
            spec_k = ctx.fft2d(np.ascontiguousarray(w[None]), spec.ax, spec.by, +1)[0]
            write_cbed(f"{stem}_diffraction_{th:g}A.cbed", spec_k, spec.ax, spec.by, th, kev)
        waves.append(w)
    results["waves"] = waves
    return results


def run_job_file(path, device=0):
    """Run a reference job file; the root tag selects the front end."""
    root = ET.parse(path).getroot()
    base = os.path.dirname(os.path.abspath(path))
    with Context(device) as ctx:
        if root.tag == "action":
            return run_lmultislice(root, base, ctx)
        if root.tag == "Calculation_parameters":
            return run_musli(root, base, ctx)
    raise ValueError(f"unknown job file root <{root.tag}>")
