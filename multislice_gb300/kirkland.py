"""Kirkland's mulslice front end: layer potentials in floatTIFF files, a
stacking sequence such as "20(ab)c", and the exit wave (or CTEM image) written
back as a floatTIFF file, with the slice loop on the GPU.

* parlay(): the stacking-sequence grammar of slicelib.cpp:558-720 -- layer
  letters a..z A..Z, a repeat count n(...) that may nest, blanks ignored, the
  reference's error codes.
* mulslice(): mulslice.cpp:296-420 (read the start wave and the layers: pDX, pDY
  give the cell, pC the layer thickness, the pixels vz with phase
  lambda mm0 vz in float as there), :706-739 (slice loop, here msl_multislice),
  :744-786 (output parameters and file layout).
"""
from __future__ import annotations

import numpy as np

from . import floattiff as FT
from .api import sigma, wavelength

_NAMES = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"


class StackingError(ValueError):
    """A stacking sequence the reference's parlay() rejects; .code is its return value."""

    def __init__(self, code, msg):
        super().__init__(f"{msg} (parlay code {code})")
        self.code = code


def parlay(c, nlayer, nsmax=1 << 20):
    """0-based layer indices of a stacking sequence (slicelib.cpp:620-720)."""
    out = []
    stack = []
    ic, n = 0, len(c)
    while ic < n:
        while ic < n and c[ic].isspace():
            ic += 1
        ch = c[ic] if ic < n else "\0"
        if ch.isalpha() and ch in _NAMES:
            name = _NAMES.index(ch)
            if name > nlayer - 1:
                raise StackingError(-1, f"layer /{ch}/ out of range")
            if len(out) >= nsmax:
                raise StackingError(-7, "too many layers")
            out.append(name)
        elif ch.isdigit():
            if len(stack) >= 100:
                raise StackingError(-3, "parenthesis nested too deep")
            j = ic
            while j < n and c[j].isdigit():
                j += 1
            rep = int(c[ic:j]) - 1
            ic = j
            while ic < n and (c[ic].isdigit() or c[ic].isspace()):
                ic += 1
            if ic >= n or c[ic] != "(":
                raise StackingError(-2, "missing left parenthesis")
            stack.append((len(out), rep))
        elif ch == ")":
            if not stack:
                raise StackingError(-5, "unmatched right parenthesis")
            start, rep = stack.pop()
            block = out[start:]
            if len(out) + rep * len(block) > nsmax:
                raise StackingError(-7, "too many layers")
            out.extend(block * rep)
        else:
            raise StackingError(-6, f"invalid character /{ch}/")
        ic += 1
    if stack:
        raise StackingError(-8, "incomplete stacking sequence")
    return out


def layers_to_transmission(ctx, vz_layers, ax, by, kev):
    """Band-limited transmissions exp(i lambda mm0 vz) of mulslice's layers
    (mulslice.cpp:344-345, :414-421; float phase as there), built on the GPU by
    msl_transmission_build from the equivalent projected potential."""
    f32 = np.float32
    mm0 = f32(1.0) + f32(kev) / f32(511.0)
    scale = f32(f32(wavelength(kev)) * mm0)
    phase = (scale * np.asarray(vz_layers, np.float32)).astype(np.float32)
    v = (phase.astype(np.float64) / sigma(kev)).astype(np.float32)
    return ctx.transmission(v, ax, by, kev)


def mulslice(ctx, layer_files, stacking, kev, out_path, start_wave=None, ctilt=(0.0, 0.0), lens=None):
    """Run mulslice on the GPU: layer_files[i] is layer letter i of `stacking`.
    Writes the exit wave (or, with lens = dict(cs=, df=, k_obj=), the coherent
    CTEM image intensity) to out_path; returns (result array, layer sequence)."""
    vz, cz = [], []
    ax = by = None
    for f in layer_files:
        v, a, b, c, _ = FT.read_potential_layer(f)
        if ax is None:
            ax, by = a, b
        elif v.shape != vz[0].shape or abs(a - ax) > 1e-4 * ax or abs(b - by) > 1e-4 * by:
            raise ValueError(f"layer {f}: size or cell incompatible with the first layer")
        vz.append(v)
        cz.append(c)
    seq = parlay(stacking, len(layer_files))
    nx, ny = vz[0].shape
    t = layers_to_transmission(ctx, np.stack(vz), ax, by, kev)
    psi = None
    params = None
    if start_wave is not None:
        psi, params = FT.read_exit_wave(start_wave)
        psi = np.ascontiguousarray(psi[None])
    lam = float(np.float32(wavelength(kev)))
    if lens is not None:
        img, w, _ = ctx.ctem_image(t, np.asarray(cz, np.float64), seq, ax, by, kev, lens["cs"], lens["df"],
                                   lens["k_obj"], psi=psi)
        FT.write_image(out_path, img.astype(np.float32), ax, by, kev, lam,
                       lens=dict(defocus=lens["df"], cs=lens["cs"],
                                 oapert=lens["k_obj"] * wavelength(kev)), params=params)
        return img, seq
    w = ctx.multislice(t, np.asarray(cz, np.float64), seq, ax, by, kev, psi=psi)[0]
    FT.write_exit_wave(out_path, w, ax, by, kev, len(seq), lam, ctilt=ctilt, params=params)
    return w, seq
