"""Drop-in GPU Modules of pyMOTO's compliance path.

Each class keeps the constructor keywords and the response / sensitivity contract of its pyMOTO
counterpart and runs on the device through libpymoto_gb300.  Signal states may be numpy arrays (the
answer is then numpy, so the modules mix with pyMOTO's own modules and optimizers) or CUDA tensors
(everything stays on the device).
"""
import math
import re

import numpy as np
import torch

from ._lib import F64, call, stream
from .core import Module
from .domain import grid_of
from .operators import (Grid, ScalarOperator, StiffnessOperator, Workspace, bc_node_mask, element_mass,
                        element_poisson, element_stiffness)
from .solvers import _from_device, _to_device, default_solver


def _kind_of(v):
    if isinstance(v, torch.Tensor):
        return "torch" if v.is_cuda else "torch-cpu"
    return "numpy"


# --------------------------------------------------------------------------------------------- filters
class DensityFilter(Module):
    """y = H x / s with H_ij = max(0, r - |c_i - c_j|) (pymoto/modules/filter.py:273-378, Filter :223-270)."""

    def __init__(self, domain, radius=2.0, nonpadding=None):
        self.domain = domain
        self.grid = Grid(*grid_of(domain))
        self.radius = float(radius)
        self.nonpadding = None if nonpadding is None else np.asarray(nonpadding, dtype=np.int64).ravel()
        self._s = None

    @property
    def H(self):
        """The filter matrix as pyMOTO builds it (scipy CSC, host; pymoto/modules/filter.py:307-378), for code
        that reads it.  The device path never forms it: the kernels evaluate the weights on the fly."""
        if getattr(self, "_H", None) is None:
            import scipy.sparse as sps
            g = self.grid
            nx, ny, nz = g.nelx, g.nely, max(g.nelz, 1)
            dl = int(self.radius)
            el = np.arange(g.nel)
            ix, iy, iz = el % nx, (el // nx) % ny, el // (nx * ny)
            rows, cols, vals = [], [], []
            for dz in range(-dl, dl + 1) if g.nelz else [0]:
                for dy in range(-dl, dl + 1):
                    for dx in range(-dl, dl + 1):
                        jx, jy, jz = ix + dx, iy + dy, iz + dz
                        ok = (jx >= 0) & (jx < nx) & (jy >= 0) & (jy < ny) & (jz >= 0) & (jz < nz)
                        rows.append(el[ok])
                        cols.append((jz[ok] * ny + jy[ok]) * nx + jx[ok])
                        h = max(0.0, self.radius - np.sqrt(dx * dx + dy * dy + dz * dz))
                        vals.append(np.full(int(ok.sum()), h))
            self._H = sps.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                     shape=(g.nel, g.nel)).tocsc()
        return self._H

    @property
    def Hs(self):
        """Row sums of H (an (nel, 1) matrix, as pyMOTO's), the rows outside `nonpadding` set to their maximum."""
        hs = self.H.sum(1)
        if self.nonpadding is not None:
            hs[~np.isin(np.arange(hs.shape[0]), self.nonpadding)] = np.max(hs)
        return hs

    def _rowsum(self, device):
        """Row sums s of H on the device; with `nonpadding`, every row outside it takes max(s), which mimics
        zero densities outside the domain (pymoto/modules/filter.py:241-255).  Setup only."""
        if self._s is None or self._s.device != device:
            g = self.grid
            self._s = torch.empty(g.nel, dtype=torch.float64, device=device)
            call("pmg_density_filter_rowsum", g.nelx, g.nely, g.nelz, self.radius, self._s, stream())
            if self.nonpadding is not None:
                outside = torch.ones(g.nel, dtype=torch.bool, device=device)
                outside[torch.from_numpy(self.nonpadding).to(device)] = False
                self._s[outside] = self._s.max()
        return self._s

    def _apply(self, v, transpose):
        vd, kind = _to_device(v)
        g = self.grid
        y = torch.empty_like(vd)
        call("pmg_density_filter", int(transpose), g.nelx, g.nely, g.nelz, self.radius, self._rowsum(vd.device), vd,
             y, stream())
        return _from_device(y, kind)

    def __call__(self, x):
        return self._apply(x, False)

    def _sensitivity(self, dfdy):
        return self._apply(dfdy, True)


def _is_value(bc):
    return isinstance(bc, (int, float, np.integer, np.floating)) and not isinstance(bc, bool)


def _pad_map(n, p, low, high):
    """Padded index map of one axis as FilterConv composes it (pymoto/modules/filter.py:98-160): wrapped
    sides first, then the high side, then the low side; numeric sides pad with index 0, and their positions
    (overridden by the constant value in pyMOTO) are marked -1 here: the kernels skip them, and the constant
    value enters through FilterConv's constant field."""
    idx = np.arange(n)
    wl = p if low == "wrap" else 0
    wh = p if high == "wrap" else 0
    if wl or wh:
        idx = np.pad(idx, (wl, wh), mode="wrap")
    for side, mode in (("high", high), ("low", low)):
        if mode == "wrap":
            continue
        width = (0, p) if side == "high" else (p, 0)
        if mode in ("edge", "symmetric"):
            idx = np.pad(idx, width, mode=mode)
        elif _is_value(mode):
            idx = np.pad(idx, width, mode="constant", constant_values=0)
        else:
            raise ValueError(f"unknown padding mode {mode!r}")
    if _is_value(low):
        idx[:p] = -1
    if _is_value(high):
        idx[len(idx) - p:] = -1
    return idx.astype(np.int32)


class FilterConv(Module):
    """Density filter as a padded convolution (pymoto/modules/filter.py:8-220).

    Padding modes 'symmetric' (default), 'edge', 'wrap' or a constant value per side.  Constant sides are
    linear: the kernel skips their padded positions (index -1 in the maps) and adds the fixed field
    conv(C) of the constant values, computed once on the host with pyMOTO's override order (later sides win
    at corners); the adjoint's inverse maps omit those positions, as pyMOTO zeroes them
    (pymoto/modules/filter.py:98-160, 207-220).
    """

    def __init__(self, domain, radius=None, relative_units=True, weights=None, xmin_bc="symmetric",
                 xmax_bc="symmetric", ymin_bc="symmetric", ymax_bc="symmetric", zmin_bc="symmetric",
                 zmax_bc="symmetric"):
        self.domain = domain
        self.grid = Grid(*grid_of(domain))
        if (weights is None) == (radius is None):
            raise ValueError("Only one of arguments 'filter_radius' or 'weights' must be provided.")
        if weights is not None:
            w = np.array(weights, dtype=np.float64)
            while w.ndim < 3:
                w = w[..., None]
            if any(s % 2 == 0 for s in w.shape):
                raise ValueError("Size of weights must be uneven")
            self.weights = w
        else:
            self.set_filter_radius(radius, relative_units)
        bcs = [xmin_bc, xmax_bc, ymin_bc, ymax_bc, zmin_bc, zmax_bc]
        g = self.grid
        sizes = [g.nelx, g.nely, max(g.nelz, 1)]
        self.pad_sizes = [s // 2 for s in self.weights.shape]
        self._maps_host = [_pad_map(n, p, bcs[2 * a], bcs[2 * a + 1]) for a, (n, p) in
                           enumerate(zip(sizes, self.pad_sizes))]
        self._bcs, self._sizes = bcs, sizes
        self._const_host = self._constant_field(bcs, sizes)
        self._dev = None
        self._overrides = {}      # element -> fixed input value (override_values)
        self._fzero = None        # the same kernel with zero padding on every side
        self._ov_dev = None
        self._padded = {}         # flat position in the padding ring -> fixed value (override_padded_values)
        self._pad_dev = None

    def override_values(self, index, value):
        """Fixed input `value` at the elements that `index` selects in the (nelx, nely, nelz) element array
        (pymoto/modules/filter.py:162-182); later calls win.  Linear: y = F(x) + F0(1_S (value - x)) with F0 the
        zero-padded convolution (padding copies still read x, as in pyMOTO), and dx = F^T dy - 1_S F0^T dy
        (pyMOTO zeroes the overridden positions in the adjoint)."""
        g = self.grid
        nz = max(g.nelz, 1)
        el = np.atleast_1d(np.arange(g.nel).reshape(nz, g.nely, g.nelx).transpose(2, 1, 0)[index])
        self._set_overrides(el.ravel(), np.broadcast_to(np.asarray(value, dtype=np.float64), el.shape).ravel())

    def _set_overrides(self, elements, values):
        for e, v in zip(elements, values):
            self._overrides[int(e)] = float(v)
        if self._fzero is None:
            w = self.weights if self.grid.nelz else self.weights[:, :, 0]
            zero = dict(xmin_bc=0.0, xmax_bc=0.0, ymin_bc=0.0, ymax_bc=0.0, zmin_bc=0.0, zmax_bc=0.0)
            self._fzero = FilterConv(self.domain, weights=w, **zero)
        self._ov_dev = None

    @property
    def padded_shape(self):
        return tuple(n + 2 * p for n, p in zip(self._sizes, self.pad_sizes))

    @property
    def padded_domain(self):
        """The element grid of the padded input (pymoto/modules/filter.py:162-167)."""
        from .domain import VoxelDomain
        nx, ny, nz = (n + 2 * p for n, p in zip((self.grid.nelx, self.grid.nely, self.grid.nelz), self.pad_sizes))
        d = self.domain
        return VoxelDomain(nx, ny, nz, unitx=d.unitx, unity=d.unity, unitz=d.unitz)

    def override_padded_values(self, index, value):
        """Fixed input `value` at the positions `index` selects in the padded array (padded_shape; pymoto's
        filter.py:169-173); later calls win.  Positions inside the domain act as override_values.  Positions in
        the padding ring replace what the padding put there, a constant or a copy x[src]: the constant part
        joins the fixed field, and each copy adds -w x[src] terms to the outputs within reach, applied as a
        gather over the (few) affected outputs with its transpose for the adjoint (pyMOTO zeroes the overridden
        positions in the adjoint)."""
        if all(np.asarray(i).size == 0 for i in (index if isinstance(index, tuple) else (index,))):
            return
        ps = self.padded_shape
        pos = np.atleast_1d(np.arange(int(np.prod(ps))).reshape(ps)[index])
        vals = np.broadcast_to(np.asarray(value, dtype=np.float64), pos.shape).ravel()
        pos = pos.ravel()
        sub = np.unravel_index(pos, ps)
        inside = np.ones(pos.size, dtype=bool)
        for a in range(3):
            inside &= (sub[a] >= self.pad_sizes[a]) & (sub[a] < self.pad_sizes[a] + self._sizes[a])
        nx, ny = self._sizes[0], self._sizes[1]
        el = ((sub[2] - self.pad_sizes[2]) * ny + (sub[1] - self.pad_sizes[1])) * nx + (sub[0] - self.pad_sizes[0])
        for k in range(pos.size):   # in call order: the last value given for a position wins
            if inside[k]:
                self._set_overrides([el[k]], [vals[k]])
                self._padded.pop(int(pos[k]), None)
            else:
                self._padded[int(pos[k])] = float(vals[k])
        self._pad_dev = None
        self._dev = None

    def get_padded_vector(self, x):
        """The padded input array that pyMOTO's FilterConv convolves (pymoto/modules/filter.py:183-187), of shape
        padded_shape: padding, constant sides and overrides applied.  Numpy in, numpy out; a tensor stays on its
        device.  For inspection: the filter itself never forms this array."""
        ps, pads = self.padded_shape, self.pad_sizes
        nx, ny = self._sizes[0], self._sizes[1]
        A, B, Cz = np.meshgrid(*self._maps_host, indexing="ij")
        fixed = (A < 0) | (B < 0) | (Cz < 0)
        src = np.where(fixed, 0, (Cz.astype(np.int64) * ny + B) * nx + A)
        val = self._constant_padded(self._bcs, self._sizes)
        for e, v in self._overrides.items():
            i, j, k = e % nx, (e // nx) % ny, e // (nx * ny)
            fixed[i + pads[0], j + pads[1], k + pads[2]] = True
            val[i + pads[0], j + pads[1], k + pads[2]] = v
        for f, v in self._padded.items():
            at = np.unravel_index(f, ps)
            fixed[at], val[at] = True, v
        if isinstance(x, torch.Tensor):
            out = x.reshape(-1)[torch.from_numpy(src).to(x.device)]
            m = torch.from_numpy(fixed).to(x.device)
            out[m] = torch.from_numpy(val).to(device=x.device, dtype=x.dtype)[m]
            return out
        out = np.asarray(x).reshape(-1)[src]
        out[fixed] = val[fixed]
        return out

    def _padded_override_host(self):
        """(fixed field, rows, row table, columns, column table) of the padding-ring overrides."""
        ps, pads, sizes = self.padded_shape, self.pad_sizes, self._sizes
        kx, ky, kz = self.weights.shape
        C = self._constant_padded(self._bcs, sizes)
        mx, my, mz = self._maps_host
        nx, ny, nz = sizes
        D = np.zeros(ps)
        terms = {}   # (output element, source element) -> coefficient
        for f, v in self._padded.items():
            a, b, c = np.unravel_index(f, ps)
            src = (int(mx[a]), int(my[b]), int(mz[c]))
            if min(src) < 0:
                D[a, b, c] = v - C[a, b, c]
                continue
            D[a, b, c] = v
            j = (src[2] * ny + src[1]) * nx + src[0]
            for oz in range(max(0, c - (kz - 1)), min(nz - 1, c) + 1):
                for oy in range(max(0, b - (ky - 1)), min(ny - 1, b) + 1):
                    for ox in range(max(0, a - (kx - 1)), min(nx - 1, a) + 1):
                        wv = self.weights[ox + kx - 1 - a, oy + ky - 1 - b, oz + kz - 1 - c]
                        if wv != 0.0:
                            o = (oz * ny + oy) * nx + ox
                            terms[(o, j)] = terms.get((o, j), 0.0) - wv
        fixed = self._valid_conv(D)

        def table(pairs):
            """Unique keys and, per key, its (index, coefficient) list padded with zero coefficients."""
            if not pairs:
                return np.zeros(0, dtype=np.int64), np.zeros((0, 1), dtype=np.int64), np.zeros((0, 1))
            kq = np.array(sorted(pairs), dtype=np.int64)
            cv = np.array([pairs[(int(r), int(q))] for r, q in kq])
            keys, start, count = np.unique(kq[:, 0], return_index=True, return_counts=True)
            slot = np.arange(kq.shape[0]) - np.repeat(start, count)
            row = np.repeat(np.arange(keys.size), count)
            idx = np.zeros((keys.size, int(count.max())), dtype=np.int64)
            coef = np.zeros((keys.size, int(count.max())))
            idx[row, slot], coef[row, slot] = kq[:, 1], cv
            return keys, idx, coef
        rows = table(terms)
        cols = table({(j, o): cv for (o, j), cv in terms.items()})
        return fixed, rows, cols

    def _override_data(self, device):
        if self._ov_dev is None or self._ov_dev[0].device != device:
            idx = np.array(sorted(self._overrides), dtype=np.int64)
            val = np.array([self._overrides[i] for i in idx], dtype=np.float64)
            self._ov_dev = (torch.from_numpy(idx).to(device), torch.from_numpy(val).to(device),
                            torch.ones(1, dtype=torch.float64, device=device))
        return self._ov_dev

    @staticmethod
    def _padded_terms(y, v, data, transpose):
        """Add the padding-ring overrides' terms to y (in place): y += conv(value - pad(v)) over the overridden
        positions, or for the adjoint the removal of their copies' contributions.  Every output row is written
        once, by a fixed-order sum over its table row."""
        fixed, rows, idx_r, coef_r, cols, idx_c, coef_c = data
        if transpose:
            if cols.numel():
                y[cols] += (coef_c * v[idx_c]).sum(1)
        else:
            y += fixed
            if rows.numel():
                y[rows] += (coef_r * v[idx_r]).sum(1)
        return y

    def _padded_data(self, device):
        if self._pad_dev is None or self._pad_dev[0].device != device:
            fixed, rows, cols = self._padded_override_host()
            self._pad_dev = tuple(torch.from_numpy(np.ascontiguousarray(t)).to(device) for t in (fixed, *rows, *cols))
        return self._pad_dev

    def _constant_field(self, bcs, sizes):
        """conv(C) on the element grid (element numbering), C the padded field that holds the constant values on
        the padded slabs of constant sides and 0 elsewhere; None when no side has a nonzero constant."""
        if not any(_is_value(b) and float(b) != 0.0 for b in bcs):
            return None
        return self._valid_conv(self._constant_padded(bcs, sizes))

    def _constant_padded(self, bcs, sizes):
        """The padded field C of the constant sides' values, 0 elsewhere."""
        pads = self.pad_sizes
        C = np.zeros([n + 2 * p for n, p in zip(sizes, pads)])
        for a in range(3):   # x, y, z; high side before low side, later overrides win (filter.py:123-160)
            p, n = pads[a], sizes[a]
            for bc, rng in ((bcs[2 * a + 1], p + n + np.arange(p)), (bcs[2 * a], np.arange(p))):
                if _is_value(bc) and rng.size:
                    sl = [slice(None)] * 3
                    sl[a] = rng
                    C[tuple(sl)] = float(bc)
        return C

    def _valid_conv(self, C):
        """'valid' convolution of a padded field with the kernel, in element numbering (host, setup)."""
        sizes = self._sizes
        kx, ky, kz = self.weights.shape
        y3 = np.zeros(sizes)
        for a in range(kx):   # 'valid' convolution: output o reads C[o + (k-1) - m]
            for b in range(ky):
                for c in range(kz):
                    y3 += self.weights[a, b, c] * C[kx - 1 - a:kx - 1 - a + sizes[0], ky - 1 - b:ky - 1 - b + sizes[1],
                                                    kz - 1 - c:kz - 1 - c + sizes[2]]
        return np.ascontiguousarray(y3.transpose(2, 1, 0)).ravel()   # element (i, j, k) -> (k ny + j) nx + i

    def set_filter_radius(self, radius, relative_units=True):
        """Cone kernel max(0, r - |d|) normalised to unit sum (pymoto/modules/filter.py:189-205)."""
        d = self.domain
        dx, dy, dz = (1.0, 1.0, 1.0) if relative_units else (d.unitx, d.unity, d.unitz)
        nx, ny, nz = grid_of(d)
        ex = min(nx, int((radius - 1e-10 * dx) / dx))
        ey = min(ny, int((radius - 1e-10 * dy) / dy))
        ez = min(nz, int((radius - 1e-10 * dz) / dz))
        X, Y, Z = np.meshgrid(np.arange(-ex, ex + 1) * dx, np.arange(-ey, ey + 1) * dy, np.arange(-ez, ez + 1) * dz,
                              indexing="ij")
        w = np.maximum(0.0, radius - np.sqrt(X * X + Y * Y + Z * Z))
        w = w / np.sum(w)
        if getattr(self, "_maps_host", None) is not None:
            # a new radius after construction: the padding was laid out for the kernel size given then
            if w.shape != self.weights.shape:
                raise ValueError(f"the new kernel {w.shape} does not fit the padding of {self.weights.shape}")
            self.weights = w
            self._const_host = self._constant_field(self._bcs, self._sizes)
            self._dev = None
            self._pad_dev = None
            if self._fzero is not None:
                self._fzero.weights = w.copy()
                self._fzero._dev = None
            return
        self.weights = w

    @staticmethod
    def _inverse_map(m, n):
        """(ptr, pos): the padded positions P with m[P] == j are pos[ptr[j]:ptr[j+1]]."""
        order = np.argsort(m, kind="stable").astype(np.int32)
        ptr = np.searchsorted(m[order], np.arange(n + 1)).astype(np.int32)
        return ptr, order

    def _device_data(self, device):
        if self._dev is None or self._dev[0].device != device:
            w = torch.from_numpy(np.ascontiguousarray(self.weights)).to(device)
            maps = [torch.from_numpy(m).to(device) for m in self._maps_host]
            g = self.grid
            sizes = [g.nelx, g.nely, max(g.nelz, 1)]
            inv = []
            for m, n in zip(self._maps_host, sizes):
                ptr, pos = self._inverse_map(m, n)
                inv += [torch.from_numpy(ptr).to(device), torch.from_numpy(pos).to(device)]
            const = None
            if self._const_host is not None:
                const = (torch.from_numpy(self._const_host).to(device),
                         torch.ones(1, dtype=torch.float64, device=device))
            self._dev = (w, *maps, *inv, const)
        return self._dev

    def _apply(self, v, transpose):
        vd, kind = _to_device(v)
        g = self.grid
        w, px, py, pz, ixp, ixs, iyp, iys, izp, izs, const = self._device_data(vd.device)
        kx, ky, kz = self.weights.shape
        y = torch.empty_like(vd)
        if transpose:
            call("pmg_conv_filter_adjoint", g.nelx, g.nely, g.nelz, w, kx, ky, kz, ixp, ixs, iyp, iys, izp, izs, vd, y,
                 stream())
        else:
            call("pmg_conv_filter", g.nelx, g.nely, g.nelz, w, kx, ky, kz, px, py, pz, vd, y, stream())
            if const is not None:   # y += conv(C): the constant-value sides
                field, one = const
                call("pmg_axpy_ratio", F64, g.nel, y, field, one, one, 1.0, stream())
        if self._padded:
            self._padded_terms(y, vd, self._padded_data(vd.device), transpose)
        if self._overrides:
            idx, val, one = self._override_data(vd.device)
            if transpose:             # dx[S] -= (F0^T d)[S]
                t = self._fzero._apply(vd, True)
                y.index_add_(0, idx, -t.index_select(0, idx))
            else:                     # y += F0(1_S (value - x))
                d = torch.zeros_like(vd)
                d.index_copy_(0, idx, val - vd.index_select(0, idx))
                call("pmg_axpy_ratio", F64, g.nel, y, self._fzero._apply(d, False), one, one, 1.0, stream())
        return _from_device(y, kind)

    def __call__(self, x):
        return self._apply(x, False)

    def _sensitivity(self, dfdv):
        return self._apply(dfdv, True)


# --------------------------------------------------------------------------------------------- SIMP
class SIMP(Module):
    """y = xmin + (1 - xmin) x^penal, the interpolation pyMOTO's examples write as
    MathExpression("xmin + (1-xmin)*inp0^3") (pymoto/modules/generic.py:14-140)."""

    def __init__(self, xmin=1e-9, penal=3.0):
        self.xmin = float(xmin)
        self.penal = float(penal)
        self.x = None

    def __call__(self, x):
        xd, kind = _to_device(x)
        self.x = xd
        y = torch.empty_like(xd)
        call("pmg_simp", xd.numel(), self.xmin, self.penal, xd, y, None, stream())
        return _from_device(y, kind)

    def _sensitivity(self, dy):
        dd, kind = _to_device(dy)
        dx = torch.empty_like(dd)
        call("pmg_simp_backward", dd.numel(), self.xmin, self.penal, self.x, dd, dx, stream())
        return _from_device(dx, kind)


_SIMP_EXPR = re.compile(r"^\s*([0-9.eE+-]+)\s*\+\s*\(\s*1\s*-\s*([0-9.eE+-]+)\s*\)\s*\*\s*(\w+)\s*(?:\^|\*\*)\s*"
                        r"([0-9.]+)\s*$")


def _torch_functions():
    """Names sympy's default printer writes, mapped to torch (device tensors stay on the device)."""
    def nmax(*a):
        out = torch.as_tensor(a[0])
        for v in a[1:]:
            out = torch.maximum(out, torch.as_tensor(v, dtype=out.dtype, device=out.device))
        return out

    def nmin(*a):
        out = torch.as_tensor(a[0])
        for v in a[1:]:
            out = torch.minimum(out, torch.as_tensor(v, dtype=out.dtype, device=out.device))
        return out
    t = torch
    return {"sin": t.sin, "cos": t.cos, "tan": t.tan, "asin": t.asin, "acos": t.acos, "atan": t.atan,
            "atan2": t.atan2, "sinh": t.sinh, "cosh": t.cosh, "tanh": t.tanh, "asinh": t.asinh, "acosh": t.acosh,
            "atanh": t.atanh, "exp": t.exp, "log": t.log, "sqrt": t.sqrt, "Abs": t.abs, "sign": t.sign,
            "floor": t.floor, "ceiling": t.ceil, "re": t.real, "im": t.imag, "conjugate": t.conj, "Max": nmax,
            "Min": nmin, "pi": float(np.pi), "E": float(np.e)}


def _zeros_like(v):
    if isinstance(v, torch.Tensor):
        return torch.zeros_like(v)
    try:
        z = v.copy()
        z[...] = 0
        return z
    except (AttributeError, TypeError):   # a Python number or a numpy scalar
        return v * 0


class MathExpression(Module):
    """pyMOTO's MathExpression (pymoto/modules/generic.py:14-140): any sympy expression of the inputs, named
    inp0, inp1, ... or by their signal tags, with sympy's derivatives for the sensitivity.

    The SIMP interpolation "a + (1-a)*inp0^p" of an element field runs in the SIMP kernels (pmg_simp,
    pmg_simp_backward).  Any other expression is evaluated by sympy's lambdify: with numpy for numpy states (as
    pyMOTO), with torch functions for tensor states (device scalars and vectors stay on the device); the
    sensitivity sums over broadcast axes as pyMOTO does."""

    def __init__(self, expression):
        self.expression = expression
        m = _SIMP_EXPR.match(expression)
        self._simp = None
        if m is not None and float(m.group(1)) == float(m.group(2)):
            self._simp = SIMP(xmin=float(m.group(1)), penal=float(m.group(4)))
            self.xmin, self.penal = self._simp.xmin, self._simp.penal
        self._mode = None
        self._fns = {}

    def _parse(self, n):
        from sympy import lambdify
        from sympy.parsing.sympy_parser import parse_expr
        text = self.expression.replace("^", "**").lower()
        expr = parse_expr(text)
        names = [f"inp{i}" for i in range(n)]
        if self.sig_in is not None:
            rep = {}
            for i, s in enumerate(self.sig_in):
                tag = getattr(s, "tag", "")
                if tag:
                    t = tag.lower()
                    if t in names and t in text:
                        raise RuntimeError(f"Name '{t}' multiple defined")
                    rep[t] = names[i]
            expr = expr.subs(rep)
        ders = [expr.diff(v) for v in names]
        tf = _torch_functions()
        self._fns = {"numpy": (lambdify(names, expr, "numpy"), lambdify(names, ders, "numpy")),
                     "torch": (lambdify(names, expr, [tf]), lambdify(names, ders, [tf]))}

    def __call__(self, *args):
        field = len(args) == 1 and (getattr(args[0], "ndim", 0) >= 1 and
                                   (args[0].numel() if isinstance(args[0], torch.Tensor) else np.size(args[0])) > 1)
        if self._simp is not None and field:
            self._mode = "simp"
            return self._simp(args[0])       # a call with plain values: no network connection
        if not self._fns:
            self._parse(len(args))
        self._mode = "torch" if any(isinstance(a, torch.Tensor) for a in args) else "numpy"
        self.x = args
        return self._fns[self._mode][0](*args)

    def _sensitivity(self, df_dy):
        if self._mode == "simp":
            return self._simp._sensitivity(df_dy)
        dg_df = self._fns[self._mode][1](*self.x)
        out = []
        for i, xi in enumerate(self.x):
            add = df_dy * dg_df[i]
            d = _zeros_like(xi)
            if isinstance(add, torch.Tensor):
                d_complex = d.is_complex() if isinstance(d, torch.Tensor) else np.iscomplexobj(d)
                if add.is_complex() and not d_complex:
                    add = add.real
                shape_d = tuple(d.shape) if hasattr(d, "shape") else ()
                if not shape_d:
                    d = d + torch.sum(torch.as_tensor(add))
                elif tuple(add.shape) != shape_d:
                    lead = add.dim() - len(shape_d)
                    axes = list(range(lead)) + [lead + k for k in range(len(shape_d))
                                                if shape_d[k] == 1 and add.shape[lead + k] != 1]
                    red = torch.sum(add, dim=axes, keepdim=True) if axes else add
                    d = d + red.reshape(shape_d)
                else:
                    d = d + add
            else:
                if np.isrealobj(d) and np.iscomplexobj(add):
                    add = np.real(add)
                if (not hasattr(d, "__len__")) or (hasattr(d, "ndim") and d.ndim == 0):
                    d += np.sum(add)
                elif d.shape != np.shape(add):
                    add = np.asarray(add)
                    lead = add.ndim - d.ndim
                    axes = tuple(range(lead)) + tuple(lead + k for k in range(d.ndim)
                                                      if d.shape[k] == 1 and add.shape[lead + k] != 1)
                    d += np.squeeze(np.add.reduce(add, axis=axes, keepdims=True), axis=tuple(range(lead)))
                else:
                    d += add
            out.append(d)
        return out


# --------------------------------------------------------------------------------------------- dyad
class DeviceDyad:
    """Sum of outer products sum_k u_k v_k^T on the device: the dK that LinSolve passes to the assembly
    (the role of pyMOTO's DyadicMatrix, pymoto/common/dyadcarrier.py)."""

    def __init__(self, u=None, v=None, shape=None):
        self.u = list(u or [])
        self.v = list(v or [])
        n = self.u[0].numel() if self.u else 0
        self.shape = shape if shape is not None else (n, n)

    @property
    def size(self):
        return self.shape[0] * self.shape[1]

    def add_sensitivity(self, other):
        self += other
        return self

    def __iadd__(self, other):
        if isinstance(other, DeviceDyad):
            self.u += other.u
            self.v += other.v
            return self
        raise TypeError(f"cannot add {type(other).__name__} to a DeviceDyad")

    def __imul__(self, s):
        self.u = [ui * s for ui in self.u]
        return self

    def __deepcopy__(self, memo):
        # new term lists, shared vectors: a dyad only ever grows by new terms and is scaled out of place
        # (__imul__), so its vectors are never written through it
        return DeviceDyad(list(self.u), list(self.v), self.shape)

    def todense(self):
        return sum(torch.outer(a, b) for a, b in zip(self.u, self.v))


# --------------------------------------------------------------------------------------------- assembly
def _stencil_constant(add_constant, grid):
    """add_constant of a one-component operator as (its diagonal, the node-stencil layout of its other entries or
    None): host FP64 arrays of nnodes and (27 or 9, nnodes), entry (o, n) coupling node n with its neighbour at
    offset o = (dz+1)*9 + (dy+1)*3 + (dx+1).  The full stencils of the one-component operators hold any constant
    whose entries couple neighbouring nodes (convection terms on boundary faces, for instance); a constant coupling
    nodes further apart, or a non-symmetric one, raises NotImplementedError."""
    n = grid.nnodes
    if add_constant is None:
        return None, None
    import scipy.sparse as sps
    if sps.issparse(add_constant) or (not isinstance(add_constant, torch.Tensor) and np.ndim(add_constant) == 2):
        A = sps.coo_matrix(add_constant)
    elif isinstance(add_constant, torch.Tensor) and add_constant.ndim == 2:
        A = sps.coo_matrix(add_constant.detach().cpu().numpy())
    else:
        return _diagonal_constant(add_constant, n), None
    if A.shape != (n, n):
        raise ValueError(f"add_constant has shape {A.shape}, the operator {(n, n)}")
    if np.iscomplexobj(A.data):
        raise NotImplementedError("add_constant: complex constants are not supported")
    A = A.tocsr()
    A.sum_duplicates()
    A = A.tocoo()
    off = A.row != A.col
    if not np.any(A.data[off] != 0):
        return _diagonal_constant(A, n), None
    scale = np.abs(A.data).max()
    if abs(A - A.T).max() > 1e-12 * scale:
        raise NotImplementedError("add_constant: the one-component operators take a symmetric constant")
    nnx, nny = grid.nelx + 1, grid.nely + 1
    r, c, v = A.row[off], A.col[off], A.data[off]
    d = [c % nnx - r % nnx, (c // nnx) % nny - (r // nnx) % nny, c // (nnx * nny) - r // (nnx * nny)]
    if any(np.abs(x).max() > 1 for x in d):
        raise NotImplementedError("add_constant: an entry couples nodes that are not neighbours")
    o = (d[2] + 1) * 9 + (d[1] + 1) * 3 + (d[0] + 1) if grid.dim == 3 else (d[1] + 1) * 3 + (d[0] + 1)
    st = np.zeros((27 if grid.dim == 3 else 9, n))
    np.add.at(st, (o, r), v)
    on = ~off
    diag = np.zeros(n)
    np.add.at(diag, A.row[on], A.data[on])
    return diag, st


def _diagonal_constant(add_constant, n):
    """The diagonal (host FP64 vector of n) of AssembleGeneral's add_constant (pymoto/modules/assembly.py:294-295):
    a sparse or dense n x n matrix, or its diagonal as a vector; None for None.  The matrix-free operators add a
    constant diagonal (springs to ground, soft supports); other constant matrices are not supported."""
    if add_constant is None:
        return None
    import scipy.sparse as sps
    if sps.issparse(add_constant):
        A = sps.coo_matrix(add_constant)
        if A.shape != (n, n):
            raise ValueError(f"add_constant has shape {A.shape}, the operator {(n, n)}")
        on = A.row == A.col
        if np.any(A.data[~on] != 0):
            raise NotImplementedError("add_constant: the matrix-free operator adds a diagonal constant only")
        c = np.zeros(n, dtype=np.result_type(A.data, np.float64))
        np.add.at(c, A.row[on], A.data[on])
    else:
        a = add_constant.detach().cpu().numpy() if isinstance(add_constant, torch.Tensor) else np.asarray(add_constant)
        if a.ndim == 1 and a.size == n:
            c = a
        elif a.shape == (n, n):
            if np.any(a - np.diag(np.diagonal(a)) != 0):
                raise NotImplementedError("add_constant: the matrix-free operator adds a diagonal constant only")
            c = np.diagonal(a)
        else:
            raise ValueError(f"add_constant has shape {a.shape}, the operator {(n, n)}")
    if np.iscomplexobj(c):
        raise NotImplementedError("add_constant: complex constants are not supported")
    return np.ascontiguousarray(c, dtype=np.float64)


class AssembleStiffness(Module):
    """K(x) = sum_e x_e K0 with Dirichlet rows/columns (pymoto/modules/assembly.py:407-463 over
    AssembleGeneral :18-315).  The output is a matrix-free StiffnessOperator on the device, not a CSR
    matrix; its sensitivity contracts the incoming dyad with K0 per element."""

    def __init__(self, domain, bc=None, bcdiagval=None, matrix_type=None, add_constant=None, reuse_sparsity=True,
                 e_modulus=1.0, poisson_ratio=0.3, plane="strain", sensitivity_precision="fp64"):
        """sensitivity_precision: "fp64" (the reference's contraction) or "mixed" (element vectors shifted
        in FP64 by their first-node value, quadratic form in FP32: for the mixed-precision solver path).
        add_constant: a constant diagonal (sparse or dense matrix, or vector) added after the Dirichlet rows."""
        if sensitivity_precision not in ("fp64", "mixed"):
            raise ValueError("sensitivity_precision must be 'fp64' or 'mixed'")
        self.sensitivity_precision = sensitivity_precision
        self.domain = domain
        self.grid = Grid(*grid_of(domain))
        g = self.grid
        self.E, self.nu, self.plane = e_modulus, poisson_ratio, plane
        unit = (domain.unitx, domain.unity, domain.unitz)
        self.stiffness_element = element_stiffness(g.dim, e_modulus, poisson_ratio, plane, unit)
        self.bc = None if bc is None else np.asarray(bc, dtype=np.int64).ravel()
        self.bcdiagval = float(np.max(self.stiffness_element)) if bcdiagval is None else float(bcdiagval)
        self._mask_host = bc_node_mask(g.nnodes, g.dim, self.bc)
        self._mask = None
        self._set_constant(add_constant, scalar=False)

    def _set_constant(self, add_constant, scalar):
        """Host diagonal of add_constant over the operator's dofs (one per node for one-component operators)."""
        g = self.grid
        self._cdiag_host = _diagonal_constant(add_constant, g.nnodes if scalar else g.ndof)
        self._cdiag = None

    def cdiag(self, device):
        if self._cdiag_host is None:
            return None
        if self._cdiag is None or self._cdiag.device != device:
            self._cdiag = torch.from_numpy(self._cdiag_host).to(device)
        return self._cdiag

    def bcmask(self, device):
        if self._mask is None or self._mask.device != device:
            self._mask = torch.from_numpy(self._mask_host).to(device)
        return self._mask

    def __call__(self, x):
        xd, kind = _to_device(x)
        if xd.numel() != self.grid.nel:
            raise ValueError(f"Input vector wrong size ({xd.numel()}), must be equal to #nel ({self.grid.nel})")
        self._kind = kind
        return StiffnessOperator(self.grid, xd, self.stiffness_element, self.bcmask(xd.device), self.bcdiagval,
                                 cdiag=self.cdiag(xd.device))

    def _sensitivity(self, dgdmat):
        if dgdmat is None or getattr(dgdmat, "size", 1) <= 0:
            return [None]
        g = self.grid
        device = self._mask.device
        dx = torch.zeros(g.nel, dtype=torch.float64, device=device)
        if isinstance(dgdmat, DeviceDyad) or (hasattr(dgdmat, "u") and hasattr(dgdmat, "v")):
            pairs = list(zip(dgdmat.u, dgdmat.v))
        else:
            raise TypeError(f"unsupported sensitivity type {type(dgdmat).__name__} (a dyad is expected)")
        for k, (u, v) in enumerate(pairs):
            ud = _to_device(u, device=device)[0]
            vd = _to_device(v, device=device)[0]
            fn = "pmg_sens_contract" if self.sensitivity_precision == "fp64" else "pmg_sens_contract_mixed"
            call(fn, g.nelx, g.nely, g.nelz, self.stiffness_element, self._mask, ud, vd, 1.0,
                 int(k > 0), dx, stream())
        return _from_device(dx, self._kind)


class _AssembleScalar(AssembleStiffness):
    """Assembly of a one-component matrix (one dof per node) as a ScalarOperator: products, multigrid and solvers
    on one value per node.  The element matrix is self.scalar_element; bc lists constrained nodes."""

    def _scalar_setup(self, domain, bc, bcdiagval, add_constant, element):
        self.domain = domain
        self.grid = Grid(*grid_of(domain))
        self.scalar_element = element
        self.bc = None if bc is None else np.asarray(bc, dtype=np.int64).ravel()
        self.bcdiagval = float(bcdiagval)
        self._mask_host = bc_node_mask(self.grid.nnodes, 1, self.bc)
        self._mask = None
        self._cdiag_host, self._cstencil_host = _stencil_constant(add_constant, self.grid)
        self._cdiag = self._cstencil = None
        if self._cstencil_host is not None and np.any(self._cstencil_host[:, self._mask_host != 0] != 0):
            # LinSolve solves Dirichlet rows directly, which needs them (and, by symmetry, their columns) free of
            # couplings
            raise NotImplementedError("add_constant: off-diagonal entries on constrained nodes are not supported")

    def cstencil(self, device):
        if self._cstencil_host is None:
            return None
        if self._cstencil is None or self._cstencil.device != device:
            self._cstencil = torch.from_numpy(self._cstencil_host).to(device)
        return self._cstencil

    def __call__(self, x):
        xd, kind = _to_device(x)
        if xd.numel() != self.grid.nel:
            raise ValueError(f"Input vector wrong size ({xd.numel()}), must be equal to #nel ({self.grid.nel})")
        self._kind = kind
        return ScalarOperator.assemble(self.grid, xd, self.scalar_element, self.bcmask(xd.device), self.bcdiagval,
                                       cdiag=self.cdiag(xd.device), cstencil=self.cstencil(xd.device))

    def _sensitivity(self, dgdmat):
        if dgdmat is None or getattr(dgdmat, "size", 1) <= 0:
            return [None]
        g = self.grid
        device = self._mask.device
        dx = torch.zeros(g.nel, dtype=torch.float64, device=device)
        if not (isinstance(dgdmat, DeviceDyad) or (hasattr(dgdmat, "u") and hasattr(dgdmat, "v"))):
            raise TypeError(f"unsupported sensitivity type {type(dgdmat).__name__} (a dyad is expected)")
        for k, (u, v) in enumerate(zip(dgdmat.u, dgdmat.v)):
            ud = _to_device(u, device=device)[0]
            vd = _to_device(v, device=device)[0]
            call("pmg_scalar_sens", g.nelx, g.nely, g.nelz, self.scalar_element, self._mask, ud, vd, 1.0, int(k > 0),
                 dx, stream())
        return _from_device(dx, self._kind)


class AssembleMass(_AssembleScalar):
    """M(x) = sum_e x_e M0 with the consistent element mass matrix (pymoto/modules/assembly.py:466-520).
    ndof = 1 (pyMOTO's default): a one-component ScalarOperator (bc: constrained nodes).  ndof = dim: the
    element matrix over dim dofs per node, as the matrix-free operator of the stiffness (bc: constrained dofs).
    Dirichlet rows and columns hold bcdiagval (default 0, as in pyMOTO).  The sensitivity is the FP64
    contraction u_e^T M0 v_e."""

    def __init__(self, domain, bc=None, bcdiagval=0.0, matrix_type=None, add_constant=None, reuse_sparsity=True,
                 material_property=1.0, ndof=1):
        g = Grid(*grid_of(domain))
        if ndof not in (1, g.dim):
            raise NotImplementedError(f"AssembleMass on the device takes ndof=1 or ndof={g.dim} (got {ndof})")
        self.ndof = ndof
        self.sensitivity_precision = "fp64"     # the mixed contraction needs an element matrix that
        self.material_property = material_property   # annihilates translations; M0 does not
        self.el_mat = element_mass(domain, ndof, material_property)
        if ndof == 1:
            self._scalar_setup(domain, bc, bcdiagval, add_constant, self.el_mat)
            return
        self.domain = domain
        self.grid = g
        self.stiffness_element = self.el_mat      # the operator's element matrix
        self.bc = None if bc is None else np.asarray(bc, dtype=np.int64).ravel()
        self.bcdiagval = float(bcdiagval)
        self._mask_host = bc_node_mask(g.nnodes, g.dim, self.bc)
        self._mask = None
        self._set_constant(add_constant, scalar=False)

    def __call__(self, x):
        if self.ndof == 1:
            return super().__call__(x)
        return AssembleStiffness.__call__(self, x)

    def _sensitivity(self, dgdmat):
        if self.ndof == 1:
            return super()._sensitivity(dgdmat)
        return AssembleStiffness._sensitivity(self, dgdmat)


class AssemblePoisson(_AssembleScalar):
    """P(x) = sum_e x_e P0 of one scalar per node (thermal conductivity, permittivity; pyMOTO's AssemblePoisson,
    pymoto/modules/assembly.py:523-560), as a one-component ScalarOperator: node stencils of 27 (3D) or 9 (2D)
    values, the same multigrid and solvers as the stiffness.  bc: constrained nodes; Dirichlet rows and columns
    hold bcdiagval (default: the largest entry of P0, as pyMOTO)."""

    def __init__(self, domain, bc=None, bcdiagval=None, matrix_type=None, add_constant=None, reuse_sparsity=True,
                 material_property=1.0):
        self.material_property = material_property
        self.poisson_element = element_poisson(domain, material_property)
        diag = float(np.max(self.poisson_element)) if bcdiagval is None else float(bcdiagval)
        self._scalar_setup(domain, bc, diag, add_constant, self.poisson_element)


# --------------------------------------------------------------------------------------------- LinSolve
class LinSolve(Module):
    """Solve K u = f (pymoto/modules/linalg.py:121-219) with the bookkeeping of the linear-dependency-aware
    wrapper that pyMOTO puts around every solver (pymoto/solvers/solvers.py:99-306):
      * Dirichlet rows (diagonal-only) are solved directly as f / bcdiag;
      * the solve starts from the previous solution with those rows zeroed (warm start);
      * each solution is stored as a normalised (u, K u) pair; later right-hand sides (the adjoint) are
        first projected on the stored pairs and only solved for when the projection residual exceeds
        5 x the solver tolerance -- so the compliance adjoint costs one FP64 residual, not a solve.
    """

    use_lda_solver = True

    def __init__(self, dep_tol=1e-5, hermitian=None, symmetric=None, positive_definite=None, solver=None):
        self.dep_tol = dep_tol
        self.ishermitian = hermitian
        self.issymmetric = symmetric
        self.ispositivedefinite = positive_definite
        self.solver = solver
        self.u = None
        self._pairs = []

    @property
    def lda_tol(self):
        return 5.0 * self.solver.tol if hasattr(self.solver, "tol") else 1e-7

    def state_dict(self):
        """The previous solution, the warm start of the next solve (checkpoint)."""
        return {"u": self.u}

    def load_state_dict(self, sd):
        self.u = sd["u"]

    def _split(self, A, rhs):
        """(direct part on Dirichlet dofs, rhs with those dofs zeroed)."""
        direct = torch.empty_like(rhs)
        rl = torch.empty_like(rhs)
        call("pmg_split_bc", F64, getattr(A, "ncomp", A.grid.dim), A.grid.nnodes, A.bcmask, A.bcdiag, rhs, direct, rl,
             A.cdiag() if hasattr(A, "cdiag") else None, stream())
        return direct, rl

    def _mask(self, A, v):
        out = torch.empty_like(v)
        call("pmg_mask_bc", F64, getattr(A, "ncomp", A.grid.dim), A.grid.nnodes, A.bcmask, 0, v, out, stream())
        return out

    def _lda_solve(self, rhs, x0=None):
        A = self.A
        ws = Workspace.get(rhs.device)
        st = stream()
        n = rhs.numel()
        sol, rl = self._split(A, rhs)
        sc = torch.zeros(4, dtype=torch.float64, device=rhs.device)
        # projection coefficients stay on the device (num / den, zero for a zero pair): no host round trip
        for xs, bs in self._pairs:   # modified Gram-Schmidt projection on the stored pairs
            call("pmg_dot2", F64, n, rl, bs, bs, bs, sc[0:1], ws.reduce, st)
            call("pmg_axpy_ratio", F64, n, rl, bs, sc[0:1], sc[1:2], -1.0, st)
            call("pmg_axpy_ratio", F64, n, sol, xs, sc[0:1], sc[1:2], 1.0, st)
        self.last_rtol = None
        if self._pairs:
            # residual of the projection: the stored pairs satisfy b_s = A x_s, so rhs - A sol is exactly the
            # projected right-hand side rl (no operator product needed).  Without stored pairs the solver's own
            # initial residual test decides.
            call("pmg_dot2", F64, n, rl, rl, rhs, rhs, sc[2:3], ws.reduce, st)
            rn, bn = (math.sqrt(max(v, 0.0)) for v in sc[2:4].tolist())
            rtol = rn / (bn if bn != 0 else 1.0)
            self.last_rtol = rtol
            if rtol <= self.lda_tol:
                return sol
        x0l = None
        if x0 is not None:
            x0l = self._mask(A, x0)
            for xs, _ in self._pairs:
                call("pmg_dot2", F64, n, x0l, xs, xs, xs, sc[0:1], ws.reduce, st)
                call("pmg_axpy_ratio", F64, n, x0l, xs, sc[0:1], sc[1:2], -1.0, st)
        xnew = self.solver.solve(rl, x0=x0l)
        xnew = self._mask(A, xnew)
        sol.add_(xnew)
        # store the new (x, A x) pair, orthogonalised against the stored ones and normalised on the device; a
        # solver that finished with an explicit FP64 residual r = rl - A xnew gives A xnew = rl - r without a
        # product
        r_fin = getattr(self.solver, "final_residual", None)
        if r_fin is not None and r_fin.shape == rl.shape and r_fin.dtype == rl.dtype:
            ba = self._mask(A, rl - r_fin)
        else:
            ba = self._mask(A, A.matvec(xnew))
        xa = xnew
        for xs, bs in self._pairs:
            call("pmg_dot2", F64, n, ba, bs, bs, bs, sc[0:1], ws.reduce, st)
            call("pmg_axpy_ratio", F64, n, ba, bs, sc[0:1], sc[1:2], -1.0, st)
            call("pmg_axpy_ratio", F64, n, xa, xs, sc[0:1], sc[1:2], -1.0, st)
        call("pmg_dot", F64, n, ba, ba, sc[2:3], ws.reduce, st)
        xn, bnv = torch.empty_like(xa), torch.empty_like(ba)
        call("pmg_scale_rsqrt", F64, n, xn, xa, sc[2:3], st)    # zero (a harmless pair) when ||ba|| is 0
        call("pmg_scale_rsqrt", F64, n, bnv, ba, sc[2:3], st)
        self._pairs.append((xn, bnv))
        return sol

    def __call__(self, mat, rhs):
        if not isinstance(mat, (StiffnessOperator, ScalarOperator)):
            raise TypeError("LinSolve on the GPU path expects the operator of AssembleStiffness, AssemblePoisson "
                            "or AssembleMass")
        fd, kind = _to_device(rhs, device=mat.device)
        self._kind = kind
        if self.solver is None:
            self.solver = default_solver(mat)
        self.solver.update(mat)
        # FP64 products of the LDA bookkeeping use the solver's (persistent, already assembled) operator
        sa = getattr(self.solver, "A64", None) or getattr(self.solver, "A", None)
        self.A = sa if type(sa) is type(mat) and sa.code == F64 else mat.astype(F64)
        self._pairs = []
        x0 = None if self.u is None else _to_device(self.u, device=mat.device)[0]
        u = self._lda_solve(fd, x0)
        self._u_dev = u
        self.u = _from_device(u, kind)
        return self.u

    def _sensitivity(self, dfdv):
        dd, kind = _to_device(dfdv, device=self._u_dev.device)
        # an adjoint solve: a solver's learned warm start (trained on the responses to the design's load) stays
        # out of it
        active = getattr(self.solver, "warm_start_active", None)
        if active is not None:
            self.solver.warm_start_active = False
        try:
            lam = self._lda_solve(dd)
        finally:
            if active is not None:
                self.solver.warm_start_active = active
        dmat = DeviceDyad([-lam], [self._u_dev])
        return dmat, _from_device(lam, kind)


# --------------------------------------------------------------------------------------------- EinSum
class EinSum(Module):
    """pyMOTO's EinSum (pymoto/modules/generic.py:143-226).  The contractions of the compliance path, 'i,i->'
    (c = f.u) and 'i->' (sum, e.g. the volume), run in the FP64 dot kernel; any other expression is evaluated
    by torch.einsum for tensor states (on their device) or numpy.einsum for numpy states, with pyMOTO's adjoint
    expressions for the sensitivities (repeated indices only in the one-input scalar form, as pyMOTO)."""

    _KERNEL = {"i,i->", "i->"}

    def __init__(self, expression):
        self.expression = expression
        expr = expression.replace(" ", "")
        self.expr = expr
        cmd = expr.split("->")
        self.indices_in = cmd[0].split(",")
        self.indices_out = cmd[1] if "->" in expr else ""
        self._general = expr not in self._KERNEL

    def _einsum(self, spec, *ops):
        if self._torch:
            return torch.einsum(spec, *ops)
        return np.einsum(spec, *ops, optimize=True)

    def _general_call(self, *args):
        self._torch = any(isinstance(a, torch.Tensor) for a in args)
        if self._torch:
            dev = next(a.device for a in args if isinstance(a, torch.Tensor))
            args = [a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a), device=dev) for a in args]
        self._args = args
        return self._einsum(self.expr, *args)

    def _general_sensitivity(self, df):
        """d(out)/d(operand k) contracted with df: the einsum of df and the other operands onto operand k's
        indices.  A single operand reduced to a scalar is the one case with repeated indices handled (a matrix
        trace: the identity pattern)."""
        ops = self._args
        torch_mode = self._torch
        if torch_mode and not isinstance(df, torch.Tensor):
            df = torch.as_tensor(np.asarray(df), device=ops[0].device, dtype=ops[0].dtype)
        repeated = [len(set(ix)) != len(ix) for ix in self.indices_in]
        if len(ops) == 1 and self.indices_out == "":
            a = ops[0]
            if not repeated[0]:
                pattern = torch.ones_like(a) if torch_mode else np.ones_like(a)
            elif a.ndim <= 2:
                pattern = (torch.eye(*a.shape, dtype=a.dtype, device=a.device) if torch_mode
                           else np.eye(*a.shape, dtype=a.dtype))
            else:
                raise NotImplementedError(f"EinSum '{self.expr}': a trace over more than two dimensions has "
                                          "no sensitivity here")
            return df * pattern
        if any(repeated):
            raise NotImplementedError(f"EinSum '{self.expr}': an operand with a repeated index has no "
                                      "sensitivity here")

        def is_complex(v):
            return v.is_complex() if torch_mode else np.iscomplexobj(v)

        grads = []
        for k, target in enumerate(self.indices_in):
            others = [(ix, v) for i, (ix, v) in enumerate(zip(self.indices_in, ops)) if i != k]
            spec = ",".join([self.indices_out] + [ix for ix, _ in others]) + "->" + target
            g = self._einsum(spec, df, *[v for _, v in others])
            # a real operand gets a real sensitivity
            grads.append(g.real if is_complex(g) and not is_complex(ops[k]) else g)
        return grads

    def __call__(self, *args):
        if self._general:
            return self._general_call(*args)
        devs = [_to_device(a) for a in args]
        self._in = devs
        ws = Workspace.get(devs[0][0].device)
        out = torch.empty(1, dtype=torch.float64, device=devs[0][0].device)
        a = devs[0][0]
        b = devs[1][0] if self.expr == "i,i->" else torch.ones_like(a)
        call("pmg_dot", F64, a.numel(), a, b, out, ws.reduce, stream())
        if all(kind == "torch" for _, kind in devs):
            return out.reshape(())      # device scalar: read by the caller when it needs the value
        return np.float64(out.item())

    def _sensitivity(self, df):
        if self._general:
            return self._general_sensitivity(df)
        df = float(df)
        if self.expr == "i->":
            (a, kind), = self._in
            return _from_device(torch.full_like(a, df), kind)
        (a, ka), (b, kb) = self._in
        da = torch.empty_like(a)
        db = torch.empty_like(b)
        call("pmg_scale", F64, b.numel(), da, b, df, stream())
        call("pmg_scale", F64, a.numel(), db, a, df, stream())
        return [_from_device(da, ka), _from_device(db, kb)]


def _sqrt(v):
    return torch.sqrt(v) if isinstance(v, torch.Tensor) else np.sqrt(v)


def _norm(v):
    return torch.linalg.vector_norm(v) if isinstance(v, torch.Tensor) else np.linalg.norm(v)


class Scaling(Module):
    """Scaling of a scalar response for the optimizers (pyMOTO's pymoto/modules/scaling.py:5-83).

    Four forms, chosen by which limits are given (s = `scaling`, a = `minmax_smooth`):
      * no limit (objective):   g = s x / |x_0|, with x_0 the value of the first response;
      * `maxval` only:          g = s (x - maxval) / |maxval|;
      * `minval` only:          g = s (minval - x) / |minval|;
      * both (smooth interval): g = s (sqrt(d^2 + a h^2) - h sqrt(1 + a)), d = x - (minval + maxval) / 2,
        h = (maxval - minval) / 2, which is <= 0 inside the interval and > 0 outside it.
    A limit of zero divides by one instead.  A device scalar (0-d CUDA tensor, e.g. EinSum's output) stays on
    the device."""

    def __init__(self, scaling: float = 100.0, minval: float = None, maxval: float = None, minmax_smooth: float = 1.0):
        self.minval, self.maxval = minval, maxval
        self.scaling, self.minmax_smooth = scaling, minmax_smooth
        if minval is not None and maxval is not None:
            self._form = "interval"
        elif maxval is not None:
            self._form = "upper"
        elif minval is not None:
            self._form = "lower"
        else:
            self._form = "objective"
        self.sf = None
        self.reset_scaling()

    @staticmethod
    def _unit(limit):
        return abs(limit) if limit != 0 else 1.0

    def _interval(self):
        return 0.5 * (self.minval + self.maxval), 0.5 * (self.maxval - self.minval)

    def __call__(self, x):
        if self.sf is None:                       # objective form: the factor is fixed by the first response
            self.sf = self.scaling / _norm(x)
        form = self._form
        if form == "objective":
            return self.sf * x
        if form == "upper":
            return self.sf * (x - self.maxval) / self._unit(self.maxval)
        if form == "lower":
            return self.sf * (self.minval - x) / self._unit(self.minval)
        mid, half = self._interval()
        a = self.minmax_smooth
        return self.sf * (_sqrt((x - mid) ** 2 + a * half ** 2) - abs(half) * np.sqrt(1.0 + a))

    def _sensitivity(self, dy):
        form = self._form
        if form == "objective":
            slope = self.sf
        elif form == "upper":
            slope = self.sf / self._unit(self.maxval)
        elif form == "lower":
            slope = -self.sf / self._unit(self.minval)
        else:
            mid, half = self._interval()
            d = self.get_input_states() - mid
            slope = self.sf * d / _sqrt(d ** 2 + self.minmax_smooth * half ** 2)
        return dy * slope

    def reset_scaling(self):
        """Forget the objective's factor (taken again from the next response); the limit forms use s itself."""
        self.sf = None if self._form == "objective" else self.scaling

    def state_dict(self):
        """The scaling factor, fixed by the first response in the objective form (checkpoint)."""
        return {"sf": self.sf}

    def load_state_dict(self, sd):
        self.sf = sd["sf"]
