"""Overhang filter, restated in numpy -- TEST INFRASTRUCTURE ONLY (the oracle of the device overhang filter).

Follows pyMOTO's OverhangFilter (pymoto/modules/filter.py:381-713) in the per-element form the device kernels
use: per layer in print order, the supports v_k of an element are the cone kernels' weighted sums of the
previous layer's printed densities (the 'valid' convolution of filter.py:647-650 written as a gather),
s = (sum_k (v_k + shift)^p)^(1/q) - backshift and y = smin(x, s); the adjoint runs the layers backwards and
returns each support derivative to the previous layer by the transposed gather (the 'full' correlation of
filter.py:707-709).  Below the first layer lies a baseplate of density 1, beside the domain zeros: at the
baseplate's lateral borders numpy's axis-by-axis padding (filter.py:634-636) leaves 1 where only axes before
the print axis are outside and 0 where an axis after it is.  Pinned against pyMOTO's outputs
(tests/golden/overhang.npz).
"""
import numpy as np


def _layer_axes(lay):
    a, b = [ax for ax in range(3) if ax != lay]
    return a, b


def _support(Y3, lay, layer_prev, kern, origin, shape):
    """v[k, ea, eb] for every element (ea, eb) of a layer whose support layer is `layer_prev` (outside the grid:
    the baseplate)."""
    a, b = _layer_axes(lay)
    na, nb = shape[a], shape[b]
    K = kern.shape[0]
    ea, eb = np.meshgrid(np.arange(na), np.arange(nb), indexing="ij")
    v = np.zeros((K, na, nb))
    base = not (0 <= layer_prev < shape[lay])
    for ma in range(kern.shape[1 + a]):
        for mb in range(kern.shape[1 + b]):
            ja = ea + origin[a] - ma
            jb = eb + origin[b] - mb
            ina = (ja >= 0) & (ja < na)
            inb = (jb >= 0) & (jb < nb)
            if base:
                # 1 unless outside in an axis padded after the print axis
                val = np.ones((na, nb))
                if a > lay:
                    val[~ina] = 0.0
                if b > lay:
                    val[~inb] = 0.0
            else:
                idx = [0, 0, 0]
                idx[lay] = layer_prev
                idx[a] = np.clip(ja, 0, na - 1)
                idx[b] = np.clip(jb, 0, nb - 1)
                val = np.where(ina & inb, Y3[tuple(idx)], 0.0)
            m = [0, 0, 0]
            m[a], m[b] = ma, mb
            w = kern[(slice(None), *m)]
            v += w[:, None, None] * val[None]
    return v


def _to3(grid, f):
    nx, ny, nz = grid
    return f.reshape(max(nz, 1), ny, nx).transpose(2, 1, 0)


def _from3(a3):
    return np.ascontiguousarray(a3.transpose(2, 1, 0)).ravel()


def overhang_forward(grid, kern, origin, lay, step, p, q, shift, backshift, eps, x):
    """(y, s): printed densities and the smooth maxima of the supports (filter.py:612-664)."""
    nx, ny, nz = grid
    shape = (nx, ny, max(nz, 1))
    X3 = _to3(grid, x)
    Y3 = np.zeros(shape)
    S3 = np.zeros(shape)
    n = shape[lay]
    for t in range(n):
        layer = t if step > 0 else n - 1 - t
        v = _support(Y3, lay, layer - step, kern, origin, shape)
        s = np.power(np.sum(np.power(v + shift, p), axis=0), 1 / q) - backshift
        sl = [slice(None)] * 3
        sl[lay] = layer
        xl = X3[tuple(sl)]
        r = xl - s
        Y3[tuple(sl)] = (xl + s - np.sqrt(r * r + eps) + np.sqrt(eps)) / 2
        S3[tuple(sl)] = s
    return _from3(Y3), _from3(S3)


def overhang_adjoint(grid, kern, origin, lay, step, p, q, shift, backshift, eps, x, y, s, dy):
    """dx from dy (filter.py:666-713), the support derivatives returned by the transposed gather."""
    nx, ny, nz = grid
    shape = (nx, ny, max(nz, 1))
    X3, Y3, S3, D3 = _to3(grid, x), _to3(grid, y), _to3(grid, s), _to3(grid, dy).copy()
    DX3 = np.zeros(shape)
    a, b = _layer_axes(lay)
    na, nb = shape[a], shape[b]
    n = shape[lay]
    for t in range(n):
        layer = n - 1 - t if step > 0 else t
        sl = [slice(None)] * 3
        sl[lay] = layer
        d = D3[tuple(sl)]
        r = X3[tuple(sl)] - S3[tuple(sl)]
        dr = -d * r / (2 * np.sqrt(r * r + eps))
        DX3[tuple(sl)] = d / 2 + dr
        ds = d / 2 - dr
        xsum = np.power(S3[tuple(sl)] + backshift, q)
        dsum = ds * np.power(xsum, 1 / q - 1) / q
        prev = layer - step
        if not (0 <= prev < n):
            continue
        v = _support(Y3, lay, prev, kern, origin, shape)
        dsupp = p * dsum[None] * np.power(v + shift, p - 1)          # [K, na, nb]
        # transposed gather: element j of the previous layer receives from o = j - origin + m
        jb_, ja_ = np.meshgrid(np.arange(nb), np.arange(na))
        acc = np.zeros((na, nb))
        for ma in range(kern.shape[1 + a]):
            for mb in range(kern.shape[1 + b]):
                oa = ja_ - origin[a] + ma
                ob = jb_ - origin[b] + mb
                ok = (oa >= 0) & (oa < na) & (ob >= 0) & (ob < nb)
                m = [0, 0, 0]
                m[a], m[b] = ma, mb
                w = kern[(slice(None), *m)]
                g = np.where(ok[None], dsupp[:, np.clip(oa, 0, na - 1), np.clip(ob, 0, nb - 1)], 0.0)
                acc += np.tensordot(w, g, axes=(0, 0))
        sp = [slice(None)] * 3
        sp[lay] = prev
        D3[tuple(sp)] += acc
    return _from3(DX3)
