"""CPU oracle of the learned coarse-slice closure -- TEST INFRASTRUCTURE ONLY.

Only tests/ and bench.py's checker leg may import this module; the product is
libmsl.so (msl_closure_* in include/msl.h).

A float64 numpy statement of the network msl_closure.cu implements -- six
complex 3x3 convolutions with periodic boundaries (1 -> 32 -> 32 -> 32 -> 32 ->
32 -> 1 channels), CReLU between them, applied to the wave divided by its RMS on a
256^2 reference grid (sqrt(sum |psi|^2 / 256^2)),
the output added back scaled -- with its loss and its gradient with respect to
every parameter.  With ``bf16=True`` it rounds to bfloat16 where the GPU stores
bfloat16 (the scaled input, the weights, every activation and every stored
activation gradient) so the two gradients can be compared closely; with
``bf16=False`` it is the exact float64 function whose gradient
tests/test_oracle_closure.py checks by finite differences.

Parameter layout (float32 in the library): per layer l with complex channel
counts (ci, co), weights [9][co][ci][2] (re, im) then bias [co][2].  Tap t is
the offset (t // 3 - 1, t % 3 - 1) in (row, column).
"""
from __future__ import annotations

import numpy as np

C = 32
LAYERS = [(1, C), (C, C), (C, C), (C, C), (C, C), (C, 1)]   # (ci, co)


def param_count():
    return sum(9 * co * ci * 2 + co * 2 for ci, co in LAYERS)


def split_params(p):
    out, o = [], 0
    for ci, co in LAYERS:
        nw = 9 * co * ci * 2
        w = np.asarray(p[o:o + nw], np.float64).reshape(9, co, ci, 2)
        b = np.asarray(p[o + nw:o + nw + co * 2], np.float64).reshape(co, 2)
        out.append((w, b))
        o += nw + co * 2
    return out


def bf16(x):
    """Round-to-nearest-even bfloat16 of float64 values (through float32)."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def expand(w):
    """Real weights [9][2co][2ci] from complex [9][co][ci][2]: blocks [[Wr, -Wi], [Wi, Wr]]."""
    wr, wi = w[..., 0], w[..., 1]
    top = np.concatenate([wr, -wi], axis=2)
    bot = np.concatenate([wi, wr], axis=2)
    return np.concatenate([top, bot], axis=1)


def contract(dw, co, ci):
    """Complex gradient [9][co][ci][2] from the real one [9][2co][2ci]."""
    g = np.empty((9, co, ci, 2))
    g[..., 0] = dw[:, :co, :ci] + dw[:, co:, ci:]
    g[..., 1] = dw[:, co:, :ci] - dw[:, :co, ci:]
    return g


def shift(x, tap):
    """x[p + off(tap)] for x [B, H, W, ch] (periodic)."""
    dy, dx = tap // 3 - 1, tap % 3 - 1
    return np.roll(x, shift=(-dy, -dx), axis=(1, 2))


def conv(x, wreal, bias=None):
    """y[p][n] = sum_tap sum_k W[tap][n][k] x[p + off][k] (+ bias[n])."""
    y = sum(np.einsum("bhwk,nk->bhwn", shift(x, t), wreal[t]) for t in range(9))
    return y if bias is None else y + bias


def conv_t(dy, wreal):
    """Input gradient of conv: dx[q][k] = sum_tap sum_n W[tap][n][k] dy[q - off][n]."""
    return sum(np.einsum("bhwn,nk->bhwk", shift(dy, 8 - t), wreal[t]) for t in range(9))


def conv_dw(dy, x):
    """dW[tap][n][k] = sum_p dy[p][n] x[p + off][k]."""
    return np.stack([np.einsum("bhwn,bhwk->nk", dy, shift(x, t)) for t in range(9)])


def _real(z):
    """complex [B, H, W] -> real channels [B, H, W, 2]."""
    return np.stack([z.real, z.imag], axis=-1).astype(np.float64)


def forward(params, coarse, fine=None, bf=True):
    """Returns (out waves complex128 [B, H, W], loss or None, cache)."""
    rnd = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    coarse = np.asarray(coarse, np.complex128)
    B, H, W = coarse.shape
    s = np.sqrt(np.sum(np.abs(coarse) ** 2, axis=(1, 2)) / 65536.0)   # norm over a 256^2 reference area
    s = np.where(s > 0, s, 1.0).astype(np.float32).astype(np.float64)
    inv = (1.0 / s).astype(np.float32).astype(np.float64)
    layers = split_params(params)
    x = rnd(_real(coarse) * inv[:, None, None, None])
    acts = [x]
    for l, (w, b) in enumerate(layers):
        ci, co = LAYERS[l]
        wreal = rnd(expand(w))
        breal = np.concatenate([b[:, 0], b[:, 1]])
        y = conv(acts[-1], wreal, breal)
        if l < 5:
            acts.append(rnd(np.maximum(y, 0.0)))
        else:
            d = y
    out = coarse + s[:, None, None] * (d[..., 0] + 1j * d[..., 1])
    loss = None
    cache = dict(acts=acts, d=d, s=s, layers=layers, bf=bf)
    if fine is not None:
        fine = np.asarray(fine, np.complex128)
        r = (_real(fine) - _real(coarse)) / s[:, None, None, None]
        e = d - r
        loss = float(np.mean(np.sum(e * e, axis=-1)))
        cache["e"] = e
    return out, loss, cache


def gradient(params, coarse, fine, bf=True):
    """(loss, dL/dparams) in the library's parameter layout."""
    _, loss, cache = forward(params, coarse, fine, bf)
    rnd = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    acts, layers = cache["acts"], cache["layers"]
    npix = cache["e"].shape[0] * cache["e"].shape[1] * cache["e"].shape[2]
    g = 2.0 * cache["e"] / npix                       # dL/dd (FP32 on the GPU)
    grads = [None] * 6
    for l in range(5, -1, -1):
        ci, co = LAYERS[l]
        x = acts[l]
        wreal = rnd(expand(layers[l][0]))
        dwr = conv_dw(g, x)
        db = g.sum(axis=(0, 1, 2))
        grads[l] = (contract(dwr, co, ci), np.stack([db[:co], db[co:]], axis=1))
        if l > 0:
            g = rnd(conv_t(g, wreal) * (x > 0))       # stored as bf16 on the GPU
    flat = []
    for gw, gb in grads:
        flat.append(gw.ravel())
        flat.append(gb.ravel())
    return loss, np.concatenate(flat)


def init_params(seed, scale_last=0.1):
    rng = np.random.default_rng(seed)
    flat = []
    for l, (ci, co) in enumerate(LAYERS):
        sd = np.sqrt(1.0 / (9.0 * ci)) * (scale_last if l == 5 else 1.0)
        flat.append(rng.standard_normal(9 * co * ci * 2) * sd)
        flat.append(rng.standard_normal(co * 2) * 0.05)
    return np.concatenate(flat).astype(np.float32)
