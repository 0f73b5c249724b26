"""Additive-manufacturing overhang filter on the device (pyMOTO's OverhangFilter, pymoto/modules/filter.py:381-713;
Langelaar, Struct. Multidisc. Optim. 55 (2017) 871-883).

The design is printed layer by layer along an axis.  An element can print at most the smooth maximum s of its
supports, the K weighted sums v_k of the previous layer's printed densities taken by the support cone (the
elements inside the overhang angle and bilinear samples on the cone's perimeter):
    s = (sum_k (v_k + shift)^p)^(1/q) - backshift,    y = (x + s - sqrt((x - s)^2 + eps) + sqrt(eps)) / 2,
with a baseplate of density 1 below the first layer and zeros beside the domain.

Device layout: one launch per layer, one thread per element of the layer, K support kernels of the cone in the
kernel parameters.  The adjoint runs the layers backwards, one launch per layer: a thread gathers the
contributions of the later layer's support derivatives to its element (the transpose of the cone), then forms
its own element's derivatives; the support derivatives of a layer are double-buffered between launches, so no
thread writes what another reads (no atomics).
"""
import numpy as np
import torch

from ._lib import call, stream
from .core import Module
from .domain import grid_of
from .solvers import _from_device, _to_device


def _direction(val):
    """Unit print direction along one Cartesian axis, from "y", "-x", ... or a vector."""
    if isinstance(val, str):
        axes = [a for a in range(3) if "xyz"[a] in val.lower()]
        if len(axes) != 1:
            raise ValueError(f'Wrongly specified print direction {val}, should be e.g. "x", "+x", "-y"')
        v = [0.0, 0.0, 0.0]
        v[axes[0]] = -1.0 if "-" in val else 1.0
        val = v
    d = np.asarray(val, dtype=float).ravel()
    d = np.pad(d, (0, 3 - d.size)) if d.size < 3 else d[:3]
    d = d / np.linalg.norm(d)
    if np.abs(d).astype(int).sum() != 1:
        raise ValueError("The print direction must be aligned with either x, y or z directions")
    return d


def support_cone(dim, elsize, direction, angle, nsampling):
    """(kernels[K, w0, w1, w2], origin[3]) of the support cone (filter.py:498-579): direct supports are the
    window elements whose direction from the element makes at least the overhang angle with the print
    direction's reverse; perimeter supports are bilinear samples at the cone radius (two in 2D when the radius
    falls more than 1 % off an element centre, else `nsampling` around the circle)."""
    lay = int(np.argmax(np.abs(direction)))
    o1, o2 = (lay + 1) % 3, (lay + 2) % 3
    if o1 == 2 and dim == 2:
        o1, o2 = o2, o1
    step = int(np.sign(direction[lay]))
    etol = 1e-5
    h = np.asarray(elsize, dtype=float)
    ta = np.tan(np.deg2rad(angle))
    w = np.array([1, 1, 1])
    r1 = (ta - etol) * h[lay] / h[o1]
    w[o1] = int(1 + 2 * np.ceil(r1))
    if dim == 3:
        w[o2] = int(1 + 2 * np.ceil((ta - etol) * h[lay] / h[o2]))
    origin = (w - 1) // 2
    origin[lay] += step
    X = (np.arange(w[0]) - origin[0])[:, None, None] * h[0]
    Y = (np.arange(w[1]) - origin[1])[None, :, None] * h[1]
    Z = (np.arange(w[2]) - origin[2])[None, None, :] * h[2]
    with np.errstate(divide="ignore", invalid="ignore"):
        ca = (direction[0] * X + direction[1] * Y + direction[2] * Z) / np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    direct = ca <= -np.cos(np.deg2rad(angle)) + etol
    radius = h[lay] * ta
    if dim == 2 and abs(np.round(r1) - r1) > 1e-2 and nsampling >= 2:
        pts = np.zeros((2, 3))
        pts[:, lay] = -origin[lay]
        pts[0, o1], pts[1, o1] = radius, -radius
        pts[:, o2] = origin[o2]
    elif nsampling > 0:
        ang = np.linspace(0, 2 * np.pi, nsampling, endpoint=False)
        pts = np.zeros((nsampling, 3))
        pts[:, lay] = -origin[lay]
        pts[:, o1] = np.sin(ang) * radius
        pts[:, o2] = np.cos(ang) * radius
    else:
        pts = np.zeros((0, 3))
    kern = np.zeros((int(direct.sum()) + len(pts), *w))
    for k, idx in enumerate(np.argwhere(direct)):       # C order, as pyMOTO walks the window
        kern[(k, *idx)] = 1.0
    k0 = int(direct.sum())
    for k, c in enumerate(pts):
        kern[k0 + k] = (np.maximum(1 - np.abs(X - c[0]) / h[0], 0) * np.maximum(1 - np.abs(Y - c[1]) / h[1], 0) *
                        np.maximum(1 - np.abs(Z - c[2]) / h[2], 0))
    return kern, origin


def smooth_parameters(p, xi_0, nsampling, dtype=np.float64):
    """(q, shift, backshift) of the smooth maximum (filter.py:484-494): zero overshoot at xi_0, a shift that
    keeps (v + shift)^p above the smallest normal number, the backshift 5 % below the value at v = 0."""
    tiny = np.finfo(dtype).tiny
    q = p + np.log(1.0 * nsampling) / np.log(xi_0)
    shift = 100.0 * pow(tiny, 1.0 / p)
    backshift = pow(nsampling, 1 / q) * pow(shift, p / q) * 0.95
    return q, shift, backshift


class OverhangFilter(Module):
    """pyMOTO's OverhangFilter(domain, direction=(0, 1, 0), overhang_angle=45, xi_0=0.5, p=40, eps=1e-4,
    nsampling=8) on the device (FP64)."""

    def __init__(self, domain, direction=(0.0, 1.0, 0.0), overhang_angle=45.0, xi_0=0.5, p=40.0, eps=1e-4,
                 nsampling=8):
        self.domain = domain
        self.grid = grid_of(domain)
        self.dim = 2 if self.grid[2] == 0 else 3
        self.direction = _direction(direction)
        if self.dim == 2 and self.direction[2] != 0:
            raise ValueError("Z-direction must be zero for 2-dimensional domain")
        self.overhang_angle, self.xi_0, self.p, self.eps = float(overhang_angle), float(xi_0), float(p), float(eps)
        self.nsampling = min(nsampling, 2) if self.dim == 2 else nsampling
        h = (domain.unitx, domain.unity, domain.unitz)
        self.layer_offsets, self.origin = support_cone(self.dim, h, self.direction, self.overhang_angle,
                                                       self.nsampling)
        self.q, self.shift, self.backshift = smooth_parameters(self.p, self.xi_0, self.nsampling)
        self._dev = None
        self.smax = None

    def _device(self, device):
        if self._dev is None or self._dev[0].device != device:
            k = torch.from_numpy(np.ascontiguousarray(self.layer_offsets.reshape(len(self.layer_offsets), -1)))
            self._dev = (k.to(device),)
        return self._dev

    def _shape(self):
        nx, ny, nz = self.grid
        return nx, ny, max(nz, 1)

    def _args(self):
        lay = int(np.argmax(np.abs(self.direction)))
        w = self.layer_offsets.shape[1:]
        return (lay, int(np.sign(self.direction[lay])), int(w[0]), int(w[1]), int(w[2]), int(self.origin[0]),
                int(self.origin[1]), int(self.origin[2]), int(len(self.layer_offsets)))

    def __call__(self, x):
        xd, kind = _to_device(x)
        nx, ny, nz = self._shape()
        if xd.numel() != nx * ny * nz:
            raise ValueError(f"Input vector wrong size ({xd.numel()}), must be equal to #nel ({nx * ny * nz})")
        (kern,) = self._device(xd.device)
        y = torch.empty_like(xd)
        self.smax = torch.empty_like(xd)
        self._x, self._kind = xd, kind
        lay, step, w0, w1, w2, c0, c1, c2, K = self._args()
        n_layers = (nx, ny, nz)[lay]
        st = stream()
        for t in range(n_layers):
            layer = t if step > 0 else n_layers - 1 - t
            call("pmg_overhang_forward", nx, ny, nz, lay, step, layer, w0, w1, w2, c0, c1, c2, K, kern,
                 self.p, self.q, self.shift, self.backshift, self.eps, xd, y, self.smax, st)
        self._y = y
        return _from_device(y, kind)

    def _sensitivity(self, dy):
        dd = _to_device(dy, device=self._x.device)[0]
        nx, ny, nz = self._shape()
        (kern,) = self._device(dd.device)
        lay, step, w0, w1, w2, c0, c1, c2, K = self._args()
        n_layers = (nx, ny, nz)[lay]
        lsize = nx * ny * nz // n_layers
        dsupp = torch.empty((2, K, lsize), dtype=torch.float64, device=dd.device)
        dx = torch.empty_like(dd)
        st = stream()
        for t in range(n_layers):           # the layers in reverse print order
            layer = n_layers - 1 - t if step > 0 else t
            call("pmg_overhang_adjoint", nx, ny, nz, lay, step, layer, int(t == 0), w0, w1, w2, c0, c1, c2, K, kern,
                 self.p, self.q, self.shift, self.backshift, self.eps, self._x, self._y, self.smax, dd,
                 dsupp[t % 2], dsupp[(t + 1) % 2], dx, st)
        return _from_device(dx, self._kind)
