"""Device-resident stiffness operators of the multigrid hierarchy.

StiffnessOperator is what AssembleStiffness outputs in place of pyMOTO's CSR matrix
(pymoto/modules/assembly.py:245-296): the matrix-free K(x) = sum_e x_e K0 with Dirichlet rows/columns
replaced by `bcdiag` on the diagonal.  StencilOperator holds a Galerkin coarse operator R^T A R
(pymoto/solvers/iterative.py:173) as element matrices plus assembled node stencils.  ScalarOperator is the
one-component operator of AssemblePoisson and AssembleMass(ndof=1) (pymoto/modules/assembly.py:466-560) on
every level, as full node stencils.  All provide the matrix protocol the solvers use: shape, dtype, `@`,
diagonal(), T, apply().
"""
import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, MATVEC, call, stream

TORCH_DTYPE = {F64: torch.float64, F32: torch.float32}


OPERATOR_KERNELS = {"fma": 0, "tcgen05": 1}


def set_operator_kernel(kind):
    """Select the implementation of the FP32 3D level-0 operator: "fma" (FP32 FMAs on the CUDA cores, the
    default) or "tcgen05" (3xTF32 products on the tensor cores).  Returns the previous selection."""
    if kind not in OPERATOR_KERNELS:
        raise ValueError(f"operator kernel must be one of {sorted(OPERATOR_KERNELS)}")
    prev = call("pmg_set_operator_kernel", OPERATOR_KERNELS[kind])
    return {v: k for k, v in OPERATOR_KERNELS.items()}[prev]


def operator_kernel():
    """The selected implementation of the FP32 3D level-0 operator ("fma" or "tcgen05")."""
    return {v: k for k, v in OPERATOR_KERNELS.items()}[call("pmg_set_operator_kernel", -1)]


def stencil_values_per_node(dim):
    """Stored node-stencil values per node: the centre block and the forward-offset blocks of a symmetric
    operator (14 of the 27 blocks in 3D, 5 of 9 in 2D; the others are their neighbours' transposes)."""
    return (14 if dim == 3 else 5) * dim * dim


class Grid:
    """Element counts of a structured grid; nelz == 0 is 2D."""

    def __init__(self, nelx, nely, nelz=0):
        self.nelx, self.nely, self.nelz = int(nelx), int(nely), int(nelz or 0)
        self.dim = 2 if self.nelz == 0 else 3
        self.nel = self.nelx * self.nely * max(self.nelz, 1)
        self.nnodes = (self.nelx + 1) * (self.nely + 1) * (self.nelz + 1)
        self.ndof = self.nnodes * self.dim

    @property
    def dims(self):
        return self.nelx, self.nely, self.nelz

    def can_coarsen(self):
        return self.nelx % 2 == 0 and self.nely % 2 == 0 and self.nelz % 2 == 0 and self.nelx >= 2 and self.nely >= 2

    def coarse(self):
        if not self.can_coarsen():
            raise ValueError(f"grid {self.dims} must be divisible by 2")
        return Grid(self.nelx // 2, self.nely // 2, self.nelz // 2)

    def __repr__(self):
        return f"Grid{self.dims}"


class Workspace:
    """Per-device scratch for the reductions and the OC bisection (zero-filled once)."""

    _by_device = {}

    def __init__(self, device):
        self.device = device
        nred = call("pmg_reduce_scratch_bytes")
        noc = call("pmg_oc_scratch_bytes")
        self.reduce = torch.zeros(nred, dtype=torch.uint8, device=device)
        self.oc = torch.zeros(noc, dtype=torch.uint8, device=device)

    @classmethod
    def get(cls, device=None):
        device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        key = device.index if device.index is not None else torch.cuda.current_device()
        ws = cls._by_device.get(key)
        if ws is None:
            ws = cls._by_device[key] = cls(torch.device("cuda", key))
        return ws


def element_stiffness(dim, e_modulus=1.0, poisson_ratio=0.3, plane="strain", unit=(1.0, 1.0, 1.0)):
    """Element stiffness matrix of pyMOTO's AssembleStiffness, computed by the library (host)."""
    nde = (2 ** dim) * dim
    K0 = np.zeros((nde, nde))
    call("pmg_element_stiffness", dim, float(e_modulus), float(poisson_ratio), int("stress" in plane.lower()),
         float(unit[0]), float(unit[1]), float(unit[2]), K0)
    return K0


def element_mass(domain, ndof, material_property=1.0):
    """Consistent element matrix material_property * int N^T N dV with ndof components per node (pyMOTO's
    AssembleMass, pymoto/modules/assembly.py:466-520): 2x2(x2) Gauss points at +-h/(2 sqrt 3), weight
    prod(h/2); in 2D the thickness unitz multiplies the property.  Host-only, setup."""
    h = np.array([domain.unitx, domain.unity, domain.unitz], dtype=np.float64)
    dim = 2 if not domain.nelz else 3
    nn = 2 ** dim
    w = np.prod(h[:dim] / 2)
    prop = material_property * (np.prod(h[dim:]) if dim != 3 else 1.0)
    signs = [[1 if (a >> c) & 1 else -1 for c in range(3)] for a in range(nn)]
    M = np.zeros((nn * ndof, nn * ndof))
    Nmat = np.zeros((ndof, nn * ndof))
    for sg in signs:
        pos = np.array(sg) * (h / 2) / np.sqrt(3)
        N = np.ones(nn) / np.prod(h[:dim])
        for c in range(dim):
            N = N * np.array([h[c] / 2 + s2[c] * pos[c] for s2 in signs])
        for a in range(nn):
            Nmat[:, ndof * a:ndof * (a + 1)] = np.identity(ndof) * N[a]
        M += w * prop * Nmat.T @ Nmat
    return M


def element_poisson(domain, material_property=1.0):
    """Element matrix material_property * int grad N^T grad N dV of one scalar per node (pyMOTO's
    AssemblePoisson, pymoto/modules/assembly.py:523-560): 2x2(x2) Gauss points at +-h/(2 sqrt 3), weight
    prod(h/2); in 2D the thickness unitz multiplies the property.  Host-only, setup."""
    h = np.array([domain.unitx, domain.unity, domain.unitz], dtype=np.float64)
    dim = 2 if not domain.nelz else 3
    nn = 2 ** dim
    w = np.prod(h[:dim] / 2)
    prop = material_property * (h[dim:] if dim != 3 else 1.0)
    signs = [[1 if (a >> c) & 1 else -1 for c in range(3)] for a in range(nn)]
    P = np.zeros((nn, nn))
    for sg in signs:
        pos = np.array(sg) * (h / 2) / np.sqrt(3)
        B = np.ones((dim, nn)) / np.prod(h[:dim])
        for c in range(dim):
            for o in range(dim):
                if o != c:
                    B[c] = B[c] * np.array([h[o] / 2 + s2[o] * pos[o] for s2 in signs])
            B[c] = B[c] * np.array([s2[c] for s2 in signs])
        P += w * prop * B.T @ B
    return P


def bc_node_mask(nnodes, dim, bc):
    """One byte per node, bit d set for Dirichlet dof node*dim + d (host array)."""
    m = np.zeros(nnodes, dtype=np.uint8)
    if bc is not None:
        bc = np.asarray(bc, dtype=np.int64).ravel()
        if bc.size and (bc.min() < 0 or bc.max() >= nnodes * dim):
            raise IndexError("Dirichlet dof index out of range")
        np.bitwise_or.at(m, bc // dim, (1 << (bc % dim)).astype(np.uint8))
    return m


def dot(a, b, out=None, ws=None):
    """FP64 device scalar a.b (accumulated in FP64)."""
    ws = ws or Workspace.get(a.device)
    out = torch.empty(1, dtype=torch.float64, device=a.device) if out is None else out
    call("pmg_dot", _lib.dtype_code(a), a.numel(), a, b, out, ws.reduce, stream())
    return out


class _GalerkinTables:
    _cache = {}

    @classmethod
    def get(cls, K0, dim, dtype, device):
        key = (K0.tobytes(), dim, dtype, str(device))
        t = cls._cache.get(key)
        if t is None:
            nde = (2 ** dim) * dim
            host = np.zeros((2 ** dim, nde, nde))
            call("pmg_galerkin_table", dim, np.ascontiguousarray(K0, dtype=np.float64), host)
            t = cls._cache[key] = torch.from_numpy(host).to(device=device, dtype=TORCH_DTYPE[dtype])
        return t


class StiffnessOperator:
    """K(x) = sum_e x_e K0 with Dirichlet rows/columns (level 0 of the hierarchy).

    FP32 products are matrix-free: in 3D by the kernel set_operator_kernel selects (FP32 FMAs on the CUDA cores
    by default, or 3xTF32 products on the tensor cores), in 2D on the CUDA cores.  FP64 products use
    half-symmetric node stencils assembled once per operator on the first FP64 product (81 FMA per dof; the
    FP64 pipe of GB300 runs at 1/64 of the FP32 rate, so fewer FMAs win over the 549 MB of stencils at
    128x64x64) unless `fp64_stencil` is False."""

    fp64_stencil = True

    def __init__(self, grid, xe, K0, bcmask, bcdiag, dtype=F64, _xe64=None, cdiag=None):
        self.grid = grid
        self.xe = xe                      # element scaling in the operator dtype
        self.K0 = np.ascontiguousarray(K0, dtype=np.float64)
        self.bcmask = bcmask              # uint8 per node (device)
        self.bcdiag = float(bcdiag)
        # constant diagonal (ndof, FP64 device vector) added after the Dirichlet rows, or None
        self.cdiag64 = cdiag
        self._cdiag = None
        self.code = dtype
        self._xe64 = xe if _xe64 is None and dtype == F64 else _xe64
        self._diag = None
        self._variants = {dtype: self}
        self._S = None
        self.persistent = False

    @classmethod
    def like(cls, other, code):
        """An operator with its own device buffers (precision `code`) for the grid / K0 / BCs of `other`,
        meant to be refreshed in place with assign() every design iteration (stable device addresses, so
        CUDA graphs that read it stay valid)."""
        xe = torch.empty(other.xe.shape, dtype=TORCH_DTYPE[code], device=other.device)
        op = cls(other.grid, xe, other.K0, other.bcmask, other.bcdiag, code, cdiag=other.cdiag64)
        op.persistent = True
        return op

    def cdiag(self):
        """The constant diagonal in the operator's precision (None without one)."""
        if self.cdiag64 is None:
            return None
        if self._cdiag is None or self._cdiag.dtype != self.torch_dtype:
            self._cdiag = self.cdiag64 if self.code == F64 else self.cdiag64.to(self.torch_dtype)
        return self._cdiag

    def assign(self, other, derived=True):
        """Copy the element scaling of `other` (any precision) into this operator's buffer and (derived=True)
        refresh the derived stencil and diagonal in place; derived=False leaves that to refresh_derived()."""
        if other is self:
            return self
        if other.grid.dims != self.grid.dims:
            raise ValueError("assign: grid mismatch")
        src = other._xe64 if other._xe64 is not None else other.xe
        call("pmg_convert", _lib.dtype_code(src), self.code, src.numel(), src, self.xe, 1.0, stream())
        self.bcmask, self.bcdiag = other.bcmask, other.bcdiag
        if other.cdiag64 is not self.cdiag64:
            self.cdiag64, self._cdiag = other.cdiag64, None
        if derived:
            self.refresh_derived()
        return self

    def refresh_derived(self):
        """Reassemble the stencil and the diagonal (when they exist) from the current element scaling."""
        if self._S is not None:
            self._assemble_stencil(self._S)
        if self._diag is not None:
            self._diagonal_into(self._diag)
        return self

    # matrix protocol -------------------------------------------------------------------------
    @property
    def shape(self):
        return (self.grid.ndof, self.grid.ndof)

    @property
    def ndim(self):
        return 2

    @property
    def dtype(self):
        return np.dtype(np.float64 if self.code == F64 else np.float32)

    @property
    def torch_dtype(self):
        return TORCH_DTYPE[self.code]

    @property
    def device(self):
        return self.xe.device

    @property
    def T(self):
        return self

    def astype(self, code):
        """Operator with the element scaling stored in `code` precision (cached)."""
        if code in self._variants:
            return self._variants[code]
        xe = torch.empty(self.xe.shape, dtype=TORCH_DTYPE[code], device=self.xe.device)
        call("pmg_convert", self.code, code, self.xe.numel(), self.xe, xe, 1.0, stream())
        op = StiffnessOperator(self.grid, xe, self.K0, self.bcmask, self.bcdiag, code, _xe64=self._xe64,
                               cdiag=self.cdiag64)
        op._variants = self._variants
        self._variants[code] = op
        return op

    def _assemble_stencil(self, S):
        g = self.grid
        call("pmg_ebe_stencil", self.code, g.nelx, g.nely, g.nelz, self.xe, self.K0, self.bcmask, self.bcdiag, S,
             stream())
        c = self.cdiag()
        if c is not None:
            call("pmg_stencil_add_diagonal", self.code, g.nelx, g.nely, g.nelz, S, c, stream())

    def stencil(self):
        """Node stencils of this operator (assembled on first use, same precision)."""
        if self._S is None:
            g = self.grid
            self._S = torch.empty((stencil_values_per_node(g.dim), g.nnodes), dtype=self.torch_dtype,
                                  device=self.device)
            self._assemble_stencil(self._S)
        return self._S

    def cheb_step(self, u, b, dl1, d, coef, step, out):
        """Fused Chebyshev smoothing step (see Chebyshev): out = u + d with d updated from r = b - K u."""
        g = self.grid
        if self.code == F32 and g.dim == 3:
            call("pmg_ebe_cheb_step", g.nelx, g.nely, g.nelz, self.xe, self.K0, self.bcmask, self.bcdiag, u, b, dl1, d,
                 coef, step, out, self.cdiag(), stream())
            return out
        if self.code == F64 and self.fp64_stencil:
            call("pmg_stencil_cheb_step", self.code, g.nelx, g.nely, g.nelz, self.stencil(), u, b, dl1, d, coef, step,
                 out, stream())
            return out
        return None

    def apply(self, mode, u, b=None, diag=None, w=0.0, out=None):
        out = torch.empty_like(u) if out is None else out
        g = self.grid
        if self.code == F64 and self.fp64_stencil:
            call("pmg_stencil_apply", mode, self.code, g.nelx, g.nely, g.nelz, self.stencil(), u, b, diag, float(w),
                 out, stream())
        else:
            call("pmg_ebe_apply", mode, self.code, g.nelx, g.nely, g.nelz, self.xe, self.K0, self.bcmask,
                 self.bcdiag, u, b, diag, float(w), out, self.cdiag(), stream())
        return out

    def matvec(self, u, out=None):
        return self.apply(MATVEC, u, out=out)

    def __matmul__(self, u):
        if isinstance(u, np.ndarray):
            ud = torch.from_numpy(np.ascontiguousarray(u, dtype=self.dtype)).to(self.device)
            return self.__matmul__(ud).cpu().numpy()
        return self.matvec(u.contiguous())

    def _diagonal_into(self, d):
        g = self.grid
        call("pmg_ebe_diagonal", self.code, g.nelx, g.nely, g.nelz, self.xe, self.K0, self.bcmask, self.bcdiag, d,
             self.cdiag(), stream())

    def diagonal(self):
        if self._diag is None:
            self._diag = torch.empty(self.grid.ndof, dtype=self.torch_dtype, device=self.device)
            self._diagonal_into(self._diag)
        return self._diag

    def galerkin(self, out=None):
        """Coarse operator R^T K R as a StencilOperator (same precision); recomputed in place into `out`."""
        g = self.grid
        gc = g.coarse()
        nde = (2 ** g.dim) * g.dim
        table = _GalerkinTables.get(self.K0, g.dim, self.code, self.device)
        E = out.E if out is not None else torch.empty((gc.nel, nde * nde), dtype=self.torch_dtype, device=self.device)
        bl = self._constrained_coarse_elements()
        call("pmg_galerkin_from_ebe", self.code, g.nelx, g.nely, g.nelz, self.xe, self.K0,
             self.bcmask, self.bcdiag, table, bl if bl.numel() else None, int(bl.numel()), E, stream())
        cc = _restricted_diagonal(g, self.cdiag(), out)
        if out is not None:
            out.cdiag = cc
            return out.recompute()
        return StencilOperator(gc, E, self.code, cdiag=cc)

    def _constrained_coarse_elements(self):
        """Indices (int32, device) of the coarse elements with a constrained fine node; cached per BC mask."""
        key = (self.bcmask.data_ptr() if self.bcmask is not None else 0, self.grid.dims)
        cache = getattr(self, "_bclist", None)
        if cache is not None and cache[0] == key:
            return cache[1]
        g = self.grid
        gc = g.coarse()
        if self.bcmask is None:
            lst = torch.zeros(0, dtype=torch.int32, device=self.device)
        else:
            m = (self.bcmask != 0).to(torch.float32)
            if g.dim == 3:
                m = m.reshape(1, 1, g.nelz + 1, g.nely + 1, g.nelx + 1)
                hit = torch.nn.functional.max_pool3d(m, kernel_size=3, stride=2).reshape(-1)
            else:
                m = m.reshape(1, 1, g.nely + 1, g.nelx + 1)
                hit = torch.nn.functional.max_pool2d(m, kernel_size=3, stride=2).reshape(-1)
            lst = torch.nonzero(hit > 0).reshape(-1).to(torch.int32)
            assert hit.numel() == gc.nel
        self._bclist = (key, lst)
        return lst

    def __repr__(self):
        return f"StiffnessOperator({self.grid}, {self.dtype})"


def _restricted_diagonal(grid, c, out=None):
    """R^T c on the coarse grid of `grid` (the lumped Galerkin term of a constant diagonal c: R^T diag(c) R 1 =
    R^T c because the prolongation of a constant is that constant), into out.cdiag when it exists; None for
    c = None."""
    if c is None:
        return None
    gc = grid.coarse()
    buf = out.cdiag if out is not None and getattr(out, "cdiag", None) is not None else \
        torch.empty(gc.ndof, dtype=c.dtype, device=c.device)
    call("pmg_restrict", _lib.dtype_code(c), grid.nelx, grid.nely, grid.nelz, c, buf, stream())
    return buf


class StencilOperator:
    """Galerkin operator of a coarse grid: element matrices E and node stencils S (same dtype)."""

    def __init__(self, grid, E, code, cdiag=None):
        self.grid = grid
        self.E = E
        self.code = code
        self.cdiag = cdiag        # lumped constant diagonal R^T c of the level above (add_constant), or None
        g = grid
        self.S = torch.empty((stencil_values_per_node(g.dim), g.nnodes), dtype=TORCH_DTYPE[code], device=E.device)
        self._diag = None
        self.recompute()

    def recompute(self):
        """Refresh the node stencils (and the diagonal, if it was requested) from E in place."""
        g = self.grid
        call("pmg_stencil_from_elements", self.code, g.nelx, g.nely, g.nelz, self.E, self.S, stream())
        if self.cdiag is not None:
            call("pmg_stencil_add_diagonal", self.code, g.nelx, g.nely, g.nelz, self.S, self.cdiag, stream())
        if self._diag is not None:
            call("pmg_stencil_diagonal", self.code, g.nelx, g.nely, g.nelz, self.S, self._diag, stream())
        return self

    @property
    def shape(self):
        return (self.grid.ndof, self.grid.ndof)

    @property
    def dtype(self):
        return np.dtype(np.float64 if self.code == F64 else np.float32)

    @property
    def torch_dtype(self):
        return TORCH_DTYPE[self.code]

    @property
    def device(self):
        return self.E.device

    @property
    def T(self):
        return self

    def apply(self, mode, u, b=None, diag=None, w=0.0, out=None):
        out = torch.empty_like(u) if out is None else out
        g = self.grid
        call("pmg_stencil_apply", mode, self.code, g.nelx, g.nely, g.nelz, self.S, u, b, diag, float(w), out, stream())
        return out

    def cheb_step(self, u, b, dl1, d, coef, step, out):
        """Fused Chebyshev smoothing step (see Chebyshev): out = u + d with d updated from r = b - S u."""
        g = self.grid
        call("pmg_stencil_cheb_step", self.code, g.nelx, g.nely, g.nelz, self.S, u, b, dl1, d, coef, step, out,
             stream())
        return out

    def matvec(self, u, out=None):
        return self.apply(MATVEC, u, out=out)

    def __matmul__(self, u):
        if isinstance(u, np.ndarray):
            ud = torch.from_numpy(np.ascontiguousarray(u, dtype=self.dtype)).to(self.device)
            return self.matvec(ud).cpu().numpy()
        return self.matvec(u.contiguous())

    def diagonal(self):
        if self._diag is None:
            g = self.grid
            d = torch.empty(g.ndof, dtype=self.torch_dtype, device=self.device)
            call("pmg_stencil_diagonal", self.code, g.nelx, g.nely, g.nelz, self.S, d, stream())
            self._diag = d
        return self._diag

    def galerkin(self, out=None):
        g = self.grid
        gc = g.coarse()
        nde = (2 ** g.dim) * g.dim
        E = out.E if out is not None else torch.empty((gc.nel, nde * nde), dtype=self.torch_dtype, device=self.device)
        call("pmg_galerkin_from_elements", self.code, g.nelx, g.nely, g.nelz, self.E, E, stream())
        cc = _restricted_diagonal(g, self.cdiag, out)
        if out is not None:
            out.cdiag = cc
            return out.recompute()
        return StencilOperator(gc, E, self.code, cdiag=cc)

    def to_dense(self, out=None):
        g = self.grid
        A = torch.empty((g.ndof, g.ndof), dtype=torch.float64, device=self.device) if out is None else out
        call("pmg_stencil_to_dense", self.code, g.nelx, g.nely, g.nelz, self.S, A, stream())
        return A

    def bandwidth(self):
        g = self.grid
        return call("pmg_stencil_bandwidth", g.nelx, g.nely, g.nelz)

    def __repr__(self):
        return f"StencilOperator({self.grid}, {self.dtype})"


def scalar_stencil_offsets(dim):
    """Stored node-stencil values per node of a one-component operator: all 27 (3D) or 9 (2D) neighbours."""
    return 27 if dim == 3 else 9


class ScalarOperator:
    """One dof per node: pyMOTO's AssemblePoisson and AssembleMass(ndof=1) matrices
    (pymoto/modules/assembly.py:466-560), and their Galerkin coarse operators.

    The full node stencil S[o, n] (27 offsets in 3D, 9 in 2D, offset o = (dz+1)*9 + (dy+1)*3 + (dx+1)) in the
    operator precision.  Level 0 assembles it from the element scaling: S = sum_e x_e P0 in FP64, Dirichlet nodes
    (bit 0 of bcmask) with bcdiag on the diagonal only, and the constant diagonal of add_constant (cdiag, FP64
    per node) added after them (assembly.py:245-296).  Coarse levels hold R^T S R (pymoto/solvers/iterative.py:
    173), exact also for the constant diagonal.  Products read the 27 coefficients and neighbours of a node: one
    FMA per coefficient, a ninth of the FMAs of the embedded form (the scalar as the first component of a
    3-component operator)."""

    ncomp = 1

    def __init__(self, grid, S, code, bcmask=None, bcdiag=0.0, cdiag=None, xe=None, P0=None, cstencil=None):
        self.grid = grid
        self.S = S
        self.code = code
        self.bcmask = bcmask
        self.bcdiag = float(bcdiag)
        self.cdiag64 = cdiag       # FP64 device vector per node (level 0), or None
        self.cstencil = cstencil   # FP64 device stencil (offsets x nodes) of a constant's off-diagonal entries
        self.xe = xe               # FP64 element scaling of a level-0 operator (None on coarse levels)
        self.P0 = None if P0 is None else np.ascontiguousarray(P0, dtype=np.float64)
        self._variants = {code: self}
        self._cdiag = None
        self.persistent = False

    @classmethod
    def assemble(cls, grid, xe, P0, bcmask, bcdiag, cdiag=None, code=F64, cstencil=None):
        """Level-0 operator of element scaling xe (FP64 device vector); cdiag / cstencil: the diagonal and the
        neighbour couplings (FP64 stencil layout) of a constant added after the Dirichlet rows."""
        S = torch.empty((scalar_stencil_offsets(grid.dim), grid.nnodes), dtype=TORCH_DTYPE[code], device=xe.device)
        op = cls(grid, S, code, bcmask, bcdiag, cdiag, xe, P0, cstencil)
        return op.recompute()

    def recompute(self):
        """Reassemble the level-0 stencil from the element scaling, in place."""
        g = self.grid
        call("pmg_scalar_stencil", self.code, g.nelx, g.nely, g.nelz, self.xe, self.P0, self.bcmask, self.bcdiag,
             self.cdiag64, self.S, stream())
        if self.cstencil is not None:
            c = self.cstencil if self.code == F64 else self.cstencil.to(self.torch_dtype)
            if getattr(self, "_one", None) is None or self._one.device != self.S.device:
                self._one = torch.ones(1, dtype=torch.float64, device=self.S.device)
            call("pmg_axpy_ratio", self.code, self.S.numel(), self.S, c, self._one, self._one, 1.0, stream())
        return self

    @classmethod
    def like(cls, other, code):
        """An operator with its own stencil buffer (precision `code`) for the grid and BCs of `other`, refreshed in
        place with assign() (stable device addresses for captured CUDA graphs)."""
        S = torch.empty(other.S.shape, dtype=TORCH_DTYPE[code], device=other.device)
        op = cls(other.grid, S, code, other.bcmask, other.bcdiag, other.cdiag64, other.xe, other.P0, other.cstencil)
        op.persistent = True
        return op

    def assign(self, other, derived=True):
        """Copy the stencil of `other` (any precision) into this operator's buffer."""
        if other is self:
            return self
        if other.grid.dims != self.grid.dims:
            raise ValueError("assign: grid mismatch")
        call("pmg_convert", other.code, self.code, other.S.numel(), other.S, self.S, 1.0, stream())
        self.bcmask, self.bcdiag, self.xe, self.P0 = other.bcmask, other.bcdiag, other.xe, other.P0
        self.cstencil = other.cstencil
        if other.cdiag64 is not self.cdiag64:
            self.cdiag64, self._cdiag = other.cdiag64, None
        return self

    def refresh_derived(self):
        return self

    def cdiag(self):
        """The constant diagonal in the operator's precision (None without one)."""
        if self.cdiag64 is None:
            return None
        if self._cdiag is None or self._cdiag.dtype != self.torch_dtype:
            self._cdiag = self.cdiag64 if self.code == F64 else self.cdiag64.to(self.torch_dtype)
        return self._cdiag

    @property
    def shape(self):
        return (self.grid.nnodes, self.grid.nnodes)

    @property
    def ndim(self):
        return 2

    @property
    def dtype(self):
        return np.dtype(np.float64 if self.code == F64 else np.float32)

    @property
    def torch_dtype(self):
        return TORCH_DTYPE[self.code]

    @property
    def device(self):
        return self.S.device

    @property
    def T(self):
        return self

    def astype(self, code):
        """The operator with its stencil in `code` precision (cached)."""
        if code in self._variants:
            return self._variants[code]
        op = ScalarOperator.like(self, code).assign(self)
        op.persistent = False
        op._variants = self._variants
        self._variants[code] = op
        return op

    def apply(self, mode, u, b=None, diag=None, w=0.0, out=None):
        out = torch.empty_like(u) if out is None else out
        g = self.grid
        call("pmg_scalar_apply", mode, self.code, g.nelx, g.nely, g.nelz, self.S, u, b, diag, float(w), out, stream())
        return out

    def cheb_step(self, u, b, dl1, d, coef, step, out):
        return None

    def matvec(self, u, out=None):
        return self.apply(MATVEC, u, out=out)

    def __matmul__(self, u):
        if isinstance(u, np.ndarray):
            ud = torch.from_numpy(np.ascontiguousarray(u, dtype=self.dtype)).to(self.device)
            return self.matvec(ud).cpu().numpy()
        return self.matvec(u.contiguous())

    def diagonal(self):
        """The diagonal: the centre row of the stencil (a view, current after every reassembly)."""
        return self.S[scalar_stencil_offsets(self.grid.dim) // 2]

    def l1_diagonal(self, out):
        """sum_j |A_ij| per row into out: the l1-Jacobi diagonal of the Chebyshev smoother."""
        g = self.grid
        call("pmg_scalar_rowabs", self.code, g.nelx, g.nely, g.nelz, self.S, out, stream())
        return out

    def restrict(self, rf, rc):
        g = self.grid
        call("pmg_scalar_restrict", self.code, g.nelx, g.nely, g.nelz, rf, rc, stream())

    def prolong_add(self, uc, uf):
        g = self.grid
        call("pmg_scalar_prolong_add", self.code, g.nelx, g.nely, g.nelz, uc, uf, stream())

    def galerkin(self, out=None):
        """Coarse operator R^T A R (same precision); recomputed in place into `out`."""
        g = self.grid
        gc = g.coarse()
        if out is None:
            S = torch.empty((scalar_stencil_offsets(gc.dim), gc.nnodes), dtype=self.torch_dtype, device=self.device)
            out = ScalarOperator(gc, S, self.code)
            out.persistent = True
        call("pmg_scalar_galerkin", self.code, g.nelx, g.nely, g.nelz, self.S, out.S, stream())
        return out

    def to_dense(self, out=None):
        g = self.grid
        A = torch.empty((g.nnodes, g.nnodes), dtype=torch.float64, device=self.device) if out is None else out
        call("pmg_scalar_to_dense", self.code, g.nelx, g.nely, g.nelz, self.S, A, stream())
        return A

    def bandwidth(self):
        """Half bandwidth in the natural node numbering (the farthest neighbour is at offset (1, 1, 1))."""
        g = self.grid
        return 1 + (g.nelx + 1) + ((g.nelx + 1) * (g.nely + 1) if g.dim == 3 else 0)

    def __repr__(self):
        return f"ScalarOperator({self.grid}, {self.dtype})"
