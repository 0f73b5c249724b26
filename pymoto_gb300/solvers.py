"""LinearSolver plugins of the GPU path (pymoto/solvers/solvers.py:6-85 protocol: update(A), solve(rhs, x0, trans)).

  CG                  -- the block-PCG of pymoto/solvers/iterative.py:295-403 for one right-hand side, FP64
                         (or the dtype of the operator), one host read of ||r|| per iteration.
  GeometricMultigrid  -- pymoto/solvers/iterative.py:124-256: Galerkin coarse operators, damped-Jacobi
                         smoothing, V-cycle; with precision="fp32" every level runs in FP32.
  DampedJacobi        -- pymoto/solvers/iterative.py:21-47.
  DenseCholesky       -- FP64 banded Cholesky of the coarsest level (in place of SuperLU).
  MixedPrecisionCG    -- flexible CG (FCG(m)) in FP64 around an FP32 multigrid preconditioner; the
                         residual r = f - K(x) u, the operator products, the alpha/beta dot products and
                         the stopping test are FP64.
All vectors are CUDA tensors; numpy right-hand sides are accepted and answered with numpy.
"""
import math
import time
import warnings

import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, JACOBI, MATVEC, RESIDUAL, call, stream
from .domain import grid_of
from .operators import Grid, ScalarOperator, StencilOperator, StiffnessOperator, Workspace

PRECISIONS = {None: None, "fp64": F64, "float64": F64, "fp32": F32, "float32": F32}


def _to_device(v, dtype=torch.float64, device=None):
    """(tensor on the device, 'numpy' | 'torch') for a numpy array or tensor."""
    if isinstance(v, torch.Tensor):
        if v.is_cuda:
            return (v if v.dtype == dtype else v.to(dtype)).contiguous(), "torch"
        return v.to(device="cuda" if device is None else device, dtype=dtype).contiguous(), "torch-cpu"
    a = np.ascontiguousarray(np.asarray(v), dtype=np.float64 if dtype == torch.float64 else np.float32)
    return torch.from_numpy(a).to(device="cuda" if device is None else device), "numpy"


def _from_device(t, kind):
    if kind == "numpy":
        return t.cpu().numpy()
    if kind == "torch-cpu":
        return t.cpu()
    return t


class LinearSolver:
    """Base class (pymoto/solvers/solvers.py:6-85)."""

    defined = True

    def __init__(self, A=None):
        if A is not None:
            self.update(A)

    def update(self, A):
        raise NotImplementedError

    def solve(self, rhs, x0=None, trans="N"):
        raise NotImplementedError

    @staticmethod
    def residual(A, x, b, trans="N"):
        """||A x - b|| / ||b|| (FP64 on the device)."""
        xd, kind = _to_device(x)
        bd, _ = _to_device(b)
        r = A.apply(RESIDUAL, xd, bd)
        ws = Workspace.get(xd.device)
        out = torch.empty(2, dtype=torch.float64, device=xd.device)
        call("pmg_dot2", F64, r.numel(), r, r, bd, bd, out, ws.reduce, stream())
        rn, bn = (math.sqrt(max(v, 0.0)) for v in out.tolist())
        return rn / (bn if bn != 0 else 1.0)


class Preconditioner(LinearSolver):
    """Identity preconditioner (pymoto/solvers/iterative.py:11-18)."""

    def update(self, A):
        pass

    def solve(self, rhs, x0=None, trans="N"):
        return rhs.clone()


class DampedJacobi(Preconditioner):
    """z = w r / diag(A) (pymoto/solvers/iterative.py:21-47)."""

    def __init__(self, A=None, w=1.0):
        if not 0 < w <= 1:
            raise ValueError("w must be between 0 and 1")
        self.w = w
        self.D = None
        super().__init__(A)

    def update(self, A):
        self.D = A.diagonal()

    def solve(self, rhs, x0=None, trans="N"):
        out = torch.empty_like(rhs)
        call("pmg_diag_scale", _lib.dtype_code(rhs), rhs.numel(), rhs, self.D, self.w, out, stream())
        return out


class Chebyshev(Preconditioner):
    """Chebyshev polynomial smoother on the l1-Jacobi scaled operator (Saad, Iterative Methods for Sparse
    Linear Systems, Alg. 12.1; l1 smoothers: Baker, Falgout, Kolev, Yang, SIAM J. Sci. Comput. 33 (2011)).

    An extension of the reference's DampedJacobi smoother (pymoto/solvers/iterative.py:21-47): `degree`
    steps preconditioned by D_l1 = diag(sum_j |A_ij|) with the weights of the Chebyshev polynomial on
    [1/ratio, 1].  By Gershgorin's theorem the spectrum of D_l1^-1 A lies in (0, 1] for any element scaling,
    so no eigenvalue estimate is needed and no mode is amplified, however high the density contrast.  The
    l1 diagonal of a stencil operator is its row sums of |A|; for the matrix-free finest operator the
    element bound sum_e x_e sum_j |K0_aj| (>= the assembled row sum) is used.  The step coefficients live in
    device memory, so a captured V-cycle stays valid across updates.
    """

    def __init__(self, A=None, degree=2, ratio=10.0):
        if degree < 1:
            raise ValueError("degree must be >= 1")
        if not ratio > 1.0:
            raise ValueError("ratio must be > 1")
        self.degree = int(degree)
        self.ratio = float(ratio)
        self.D = None
        self.coef = None
        super().__init__(A)

    @staticmethod
    def l1_element_matrix(K0):
        """diag(sum_j |K0_aj|): fed to the diagonal kernel it yields the matrix-free l1 diagonal."""
        K0 = np.asarray(K0, dtype=np.float64)
        return np.diag(np.abs(K0).sum(axis=1))

    def update(self, A):
        n = A.shape[0]
        if self.D is None or self.D.numel() != n or self.D.dtype != A.torch_dtype or self.D.device != A.device:
            self.D = torch.empty(n, dtype=A.torch_dtype, device=A.device)
            self.coef = torch.zeros(2 * self.degree, dtype=torch.float64, device=A.device)
            call("pmg_cheb_coeffs", None, 1.0, self.ratio, self.degree, self.coef, stream())
        g = A.grid
        if isinstance(A, ScalarOperator):
            A.l1_diagonal(self.D)
        elif isinstance(A, StencilOperator):
            call("pmg_stencil_rowabs", A.code, g.nelx, g.nely, g.nelz, A.S, self.D, stream())
        else:
            # the constant diagonal (add_constant, nonnegative springs) enters the l1 row sums as it is
            call("pmg_ebe_diagonal", A.code, g.nelx, g.nely, g.nelz, A.xe, self.l1_element_matrix(A.K0), A.bcmask,
                 A.bcdiag, self.D, A.cdiag(), stream())

    def smooth(self, A, b, x, d, r, zero_start):
        """`degree` steps from x; d and r are work vectors of the size of b.  Each step is one fused
        operator product (residual, update of d and of the iterate) where the operator has it, writing the
        new iterate into the other of (x, r); returns the buffer holding the result."""
        code, n, st = A.code, b.numel(), stream()
        j0 = 0
        if zero_start:
            call("pmg_cheb_step", code, n, b, self.D, d, x, self.coef, 0, 1, st)
            j0 = 1
        cur, other = x, r
        for j in range(j0, self.degree):
            if A.cheb_step(cur, b, self.D, d, self.coef, j, out=other) is not None:
                cur, other = other, cur
            else:
                A.apply(RESIDUAL, cur, b, out=other)
                call("pmg_cheb_step", code, n, other, self.D, d, cur, self.coef, j, 0, st)
        return cur

    def solve(self, rhs, x0=None, trans="N"):
        raise NotImplementedError("Chebyshev is a multigrid smoother (GeometricMultigrid calls smooth())")


class DenseCholesky(LinearSolver):
    """Direct solve of the coarsest Galerkin operator: dense FP64 banded Cholesky on the device.

    Stands in for SolverSparseLU (pymoto/solvers/sparse.py:515-555), which auto_determine_solver picks for
    the coarse sparse matrix (pymoto/solvers/auto_determine.py:109-122).  The factorisation is always FP64.
    FP64 operators (small enough) get the explicit FP64 inverse, so that each solve is one dense product;
    FP32 operators (the mixed-precision hierarchy) get an FP32 copy of the factor and of its diagonal-tile
    inverses, and each solve is a blocked forward/backward substitution without any scalar recurrence.
    """

    MAX_DOFS = 20000
    INVERSE_MAX_DOFS = 4096   # FP64: up to this size the solve is one dense product with the explicit inverse

    def __init__(self, A=None, lag=False):
        """lag=True (FP32 operators with the explicit inverse): update() leaves the inverse of the previous
        update active and factorises the new matrix behind it (on the caller's stream, typically a side
        stream); promote_if_ready() makes the new inverse the active one as soon as it exists, so the
        factorisation runs off the critical path and a solver switches to the exact coarse solve mid-solve."""
        self.lag = lag
        self.ready_event = None
        self._pending = False
        self.L = None
        self.L32 = None
        self.Dinv32 = None
        self.Ainv = None
        self.Ainv32 = None
        super().__init__(A)

    def _ordering(self, A):
        """Band-reducing dof numbering for the explicit-inverse path (the inverse is returned to the natural
        numbering, so solves are unchanged); the blocked substitution paths keep the natural numbering."""
        g = A.grid
        if self.n > self.INVERSE_MAX_DOFS:
            return None, A.bandwidth()
        key = (g.dims, A.device, type(A))
        if getattr(self, "_order_key", None) != key and isinstance(A, ScalarOperator):
            # one dof per node: the natural numbering (its band is already that of the grid's fastest axes)
            self._pos = torch.arange(self.n, dtype=torch.int32, device=A.device)
            self._order_bw = A.bandwidth()
            self._order_key = key
        if getattr(self, "_order_key", None) != key:
            pos = np.empty(self.n, dtype=np.int32)
            bw = np.zeros(1, dtype=np.int32)
            call("pmg_coarse_ordering", g.nelx, g.nely, g.nelz, pos, bw)
            self._pos = torch.from_numpy(pos).to(A.device)
            self._order_bw = int(bw[0])
            self._order_key = key
        return self._pos, self._order_bw

    def update(self, A):
        if not isinstance(A, (StencilOperator, ScalarOperator)):
            raise TypeError("DenseCholesky expects a coarse StencilOperator or ScalarOperator")
        n = A.shape[0]
        if n > self.MAX_DOFS:
            raise ValueError(f"coarsest level has {n} dofs (> {self.MAX_DOFS}); add multigrid levels")
        self.n = n
        self.code = A.code
        pos, self.bw = self._ordering(A)
        dev = A.device
        if self.L is None or self.L.shape[0] != n or self.L.device != dev:
            # device buffers kept across updates (stable addresses for captured CUDA graphs)
            self.L = torch.empty((n, n), dtype=torch.float64, device=dev)
            self._info = torch.zeros(1, dtype=torch.int32, device=dev)
            self.Ainv = self.L32 = self.Dinv32 = self.Ainv32 = None
            self._pending = False
        lagged = self.lag and A.code == F32 and n <= self.INVERSE_MAX_DOFS
        if lagged:
            if self.ready_event is None:
                self.ready_event = torch.cuda.Event()
            if getattr(self, "Ainv32", None) is None:
                nbytes = _lib.load().pmg_cholesky_inverse_f32_scratch_bytes(n)
                self._inv_scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
                self.Ainv32 = torch.empty((n, n), dtype=torch.float32, device=dev)
                self._Ainv32_next = torch.empty((n, n), dtype=torch.float32, device=dev)
                self._pending = False
                self._have_inverse = False
                self._next_event = None
            if self._pending:                                 # never promoted: the previous update's inverse
                self.Ainv32.copy_(self._Ainv32_next)
                self._pending = False
            self.ready_event.record()
        L = self.L
        g = A.grid
        if isinstance(A, ScalarOperator):
            A.to_dense(out=L)         # natural numbering: pos is the identity
        else:
            call("pmg_stencil_to_dense_perm", A.code, g.nelx, g.nely, g.nelz, A.S, pos, L, stream())
        call("pmg_cholesky_factor", n, L, self.bw, self._info, stream())
        # the pivot check is read back without blocking the host (check() raises once it has arrived), so
        # that the host can queue the next work while the factorisation runs
        if getattr(self, "_info_host", None) is None:
            self._info_host = torch.zeros(1, dtype=torch.int32).pin_memory()
            self._info_event = torch.cuda.Event()
        self._info_host.copy_(self._info, non_blocking=True)
        self._info_event.record()
        self._checked = False
        if lagged:
            self._inverse_f32(self._Ainv32_next)
            if not self._have_inverse:                    # first update: no previous inverse to use
                self.Ainv32.copy_(self._Ainv32_next)
                self.ready_event.record()
                self._have_inverse = True
                return
            if self._next_event is None:
                self._next_event = torch.cuda.Event()
            self._next_event.record()
            self._pending = True
            return
        if A.code == F64 and n <= self.INVERSE_MAX_DOFS:
            if self.Ainv is None:
                self.Ainv = torch.empty_like(self.L)
                self._Ainv_perm = torch.empty_like(self.L)
            call("pmg_cholesky_inverse", n, L, self.bw, self._Ainv_perm, stream())
            call("pmg_dense_permute", F64, n, self._pos, self._Ainv_perm, self.Ainv, stream())
        elif A.code == F32:
            self._prepare_f32()

    def _inverse_f32(self, out):
        """FP32 inverse of the (permuted) factor, returned to the natural numbering in `out`."""
        n = self.n
        if getattr(self, "_Ainv32_perm", None) is None or self._Ainv32_perm.shape[0] != n:
            self._Ainv32_perm = torch.empty((n, n), dtype=torch.float32, device=self.L.device)
        call("pmg_cholesky_inverse_f32", n, self.L, self.bw, self._inv_scratch, self._Ainv32_perm, stream())
        call("pmg_dense_permute", F32, n, self._pos, self._Ainv32_perm, out, stream())

    def promote_if_ready(self):
        """Lagged mode: once the factorisation of the latest update has finished (checked without blocking),
        make its inverse the active one, ordered on the current stream before the solves that follow.
        Returns True when the active inverse is the current one."""
        if not self._pending:
            return True
        if not self._next_event.query():
            return False
        self.Ainv32.copy_(self._Ainv32_next)
        self._pending = False
        return True

    def check(self):
        """Raise LinAlgError if the last factorisation met a non-positive pivot (waits for the factorisation)."""
        if getattr(self, "_checked", True):
            return
        self._info_event.synchronize()
        self._checked = True
        bad = int(self._info_host.item())
        if bad != 0:
            raise np.linalg.LinAlgError(f"coarsest-level matrix not positive definite (pivot {bad - 1})")

    def _prepare_f32(self):
        n, dev = self.n, self.L.device
        if n <= self.INVERSE_MAX_DOFS:
            # explicit FP32 inverse from the FP64 factor: each solve is one dense product
            if getattr(self, "Ainv32", None) is None:
                nbytes = _lib.load().pmg_cholesky_inverse_f32_scratch_bytes(n)
                self._inv_scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
                self.Ainv32 = torch.empty((n, n), dtype=torch.float32, device=dev)
            self._inverse_f32(self.Ainv32)
            return
        if self.L32 is None:
            self.L32 = torch.empty((n, n), dtype=torch.float32, device=dev)
            self.Dinv32 = torch.empty(((n + 31) // 32) * 32 * 32, dtype=torch.float32, device=dev)
        call("pmg_convert", F64, F32, n * n, self.L, self.L32, 1.0, stream())
        call("pmg_cholesky_block_inverses", F32, n, self.L, self.Dinv32, stream())

    def solve(self, rhs, x0=None, trans="N"):
        code = _lib.dtype_code(rhs)
        out = getattr(self, "_out", None)
        if out is None or out.dtype != rhs.dtype or out.numel() != rhs.numel() or out.device != rhs.device:
            out = self._out = torch.empty_like(rhs)
        if code == F64 and self.Ainv is not None:
            call("pmg_dense_gemv", code, self.n, self.Ainv, rhs.contiguous(), out, stream())
            return out
        if code == F32:
            if getattr(self, "Ainv32", None) is None and self.L32 is None:
                self._prepare_f32()
            if getattr(self, "Ainv32", None) is not None:
                call("pmg_dense_gemv", F32, self.n, self.Ainv32, rhs.contiguous(), out, stream())
            else:
                call("pmg_cholesky_solve_blocked", F32, self.n, self.L32, self.bw, self.Dinv32, rhs.contiguous(),
                     out, stream())
            return out
        call("pmg_cholesky_solve", code, self.n, self.L, self.bw, rhs.contiguous(), out, stream())
        return out


def _restrict(A, rf, rc):
    """rc = R^T rf for the operator A of the fine level (per node for one-component operators, per dof
    component otherwise)."""
    if isinstance(A, ScalarOperator):
        A.restrict(rf, rc)
    else:
        g = A.grid
        call("pmg_restrict", A.code, g.nelx, g.nely, g.nelz, rf, rc, stream())


def _prolong_add(A, uc, uf):
    """uf += R uc for the operator A of the fine level."""
    if isinstance(A, ScalarOperator):
        A.prolong_add(uc, uf)
    else:
        g = A.grid
        call("pmg_prolong_add", A.code, g.nelx, g.nely, g.nelz, uc, uf, stream())


class GeometricMultigrid(Preconditioner):
    """Geometric multigrid preconditioner (pymoto/solvers/iterative.py:124-256).

    Galerkin coarse operator R^T A R built per coarse element on the device; V-cycle with `smooth_steps`
    damped-Jacobi sweeps before and after the coarse correction (the first pre-sweep starts from zero when
    no initial guess is given).  `precision="fp32"` runs the level (and by default its inner levels) in
    FP32 with FP32 operators; the coarsest factorisation stays FP64.
    """

    _available_cycles = ["v", "w"]

    def __init__(self, domain, A=None, cycle="V", inner_level=None, smoother=None, smooth_steps=5, precision=None):
        nx, ny, nz = grid_of(domain)
        if nx % 2 or ny % 2 or nz % 2:
            raise ValueError(f"Domain sizes {nx, ny, nz} must be divisible by 2")
        if cycle.lower() not in self._available_cycles:
            raise ValueError(f"Cycle ({cycle}) is not available. Options are {self._available_cycles}")
        self.domain = domain
        self.grid = Grid(nx, ny, nz)
        self.cycle = cycle
        self.inner_level = inner_level
        self.smoother = DampedJacobi(w=0.5) if smoother is None else smoother
        self.smooth_steps = smooth_steps
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}")
        self.precision = PRECISIONS[precision]
        self.sub_domain = type(domain)(nx // 2, ny // 2, nz // 2, domain.unitx * 2, domain.unity * 2,
                                       domain.unitz * 2)
        self.A = None
        self._buf = None
        self.use_graph = True
        self._graph = None
        super().__init__(A)

    def update(self, A):
        """Refresh the level for a new operator.  Device buffers (level-0 copy of the operator, Galerkin
        operators, diagonals, coarsest factor) are reused in place, so a captured V-cycle stays valid."""
        code = self.precision if self.precision is not None else A.code
        if isinstance(A, (StiffnessOperator, ScalarOperator)):
            if A.persistent and A.code == code:
                op = A
            else:
                a0 = getattr(self, "_A0", None)
                if a0 is None or type(a0) is not type(A) or a0.code != code or a0.grid.dims != A.grid.dims:
                    self._A0 = type(A).like(A, code)
                    self._graph = None
                op = self._A0.assign(A)
        else:
            op = A
        if op.code != code:
            raise TypeError("coarse operators keep the precision of their parent level")
        if not torch.cuda.is_current_stream_capturing():
            # the level-0 operator of this level is final here (the rest of the hierarchy follows)
            if getattr(self, "level0_ready", None) is None:
                self.level0_ready = torch.cuda.Event()
            self.level0_ready.record()
        if self.A is not op:
            self._graph = None
        self.A = op
        self.smoother.update(op)
        if getattr(self, "_Ac", None) is None or self._Ac.code != code:
            self._Ac = op.galerkin()
            self._graph = None
        else:
            op.galerkin(out=self._Ac)
        Ac = self._Ac
        if self.inner_level is None:
            self.inner_level = DenseCholesky()
        if isinstance(self.inner_level, GeometricMultigrid) and self.inner_level.precision is None:
            self.inner_level.precision = code
        self.inner_level.update(Ac)
        n = op.shape[0]
        if self._buf is None or self._buf[0].dtype != op.torch_dtype or self._buf[0].device != op.device or \
                self._buf[0].numel() != n:
            self._buf = [torch.empty(n, dtype=op.torch_dtype, device=op.device) for _ in range(3)]
            self._rc = torch.empty(Ac.shape[0], dtype=op.torch_dtype, device=op.device)

    @property
    def code(self):
        return self.A.code

    def solve(self, rhs, x0=None, trans="N"):
        """One V-cycle.  The result is a buffer of this object, valid until the next solve."""
        in_code = _lib.dtype_code(rhs)
        b = rhs if in_code == self.A.code else rhs.to(self.A.torch_dtype)
        if x0 is None and self.use_graph and not torch.cuda.is_current_stream_capturing():
            u = self._replay(b)
        else:
            u = self._vcycle(b, x0 if x0 is None or x0.dtype == b.dtype else x0.to(b.dtype))
        return u if in_code == self.A.code else u.to(rhs.dtype)

    def _replay(self, b):
        """V-cycle from a zero guess through a CUDA graph captured once per update()."""
        if self._graph is None:
            self._g_in = torch.zeros_like(b)
            self._vcycle(self._g_in)                 # eager run: loads every kernel before the capture
            graph, counter = capture_graph(lambda: self._vcycle(self._g_in))
            self._graph, self._g_out = graph, counter.result
            self._g_launches = counter.launches
        self._g_in.copy_(b)
        _lib.replay(f"vcycle{self.grid.dims}|{self.A.code}", self._graph, self._g_launches)
        return self._g_out

    def _vcycle(self, b, x0=None):
        A, w, steps = self.A, None, self.smooth_steps
        u, t, r = self._buf[0], self._buf[1], self._buf[2]
        if isinstance(self.smoother, Chebyshev):
            return self._vcycle_chebyshev(b, x0)
        fused = type(self.smoother) is DampedJacobi
        if fused:
            w, D = self.smoother.w, self.smoother.D
            n, code = b.numel(), A.code
            if x0 is None:
                call("pmg_diag_scale", code, n, b, D, w, u, stream())
            else:
                A.apply(JACOBI, x0, b, D, w, out=u)
            for _ in range(steps - 1):
                A.apply(JACOBI, u, b, D, w, out=t)
                u, t = t, u
        else:
            if x0 is None:
                u.copy_(self.smoother.solve(b))
            else:
                u.copy_(x0 + self.smoother.solve(A.apply(RESIDUAL, x0, b)))
            for _ in range(steps - 1):
                u += self.smoother.solve(A.apply(RESIDUAL, u, b, out=r))
        A.apply(RESIDUAL, u, b, out=r)
        g = self.grid
        inner = self.inner_level
        rc = self._rc
        _restrict(A, r, rc)
        uc = inner._vcycle(rc) if isinstance(inner, GeometricMultigrid) else inner.solve(rc)
        _prolong_add(A, uc, u)
        for _ in range(steps):
            if fused:
                A.apply(JACOBI, u, b, D, w, out=t)
                u, t = t, u
            else:
                u += self.smoother.solve(A.apply(RESIDUAL, u, b, out=r))
        # keep the result in the first buffer slot for the caller, swap the others
        if u.data_ptr() != self._buf[0].data_ptr():
            self._buf[0], self._buf[1] = u, self._buf[0]
        return u

    def _vcycle_chebyshev(self, b, x0=None):
        A, sm = self.A, self.smoother
        u0, u1, d = self._buf[0], self._buf[1], self._buf[2]
        if x0 is None:
            u = sm.smooth(A, b, u0, d, u1, zero_start=True)
        else:
            u0.copy_(x0)
            u = sm.smooth(A, b, u0, d, u1, zero_start=False)
        other = u1 if u is u0 else u0
        A.apply(RESIDUAL, u, b, out=other)
        g = self.grid
        inner = self.inner_level
        rc = self._rc
        _restrict(A, other, rc)
        uc = inner._vcycle(rc) if isinstance(inner, GeometricMultigrid) else inner.solve(rc)
        _prolong_add(A, uc, u)
        return sm.smooth(A, b, u, d, other, zero_start=False)

    @classmethod
    def hierarchy(cls, domain, levels=None, smoother_w=0.5, smooth_steps=5, precision=None, max_coarse_dofs=3000,
                  coarse_smooth_steps=None, smoother="jacobi", cheb_ratio=10.0, coarse_lag=False):
        """Chain of GeometricMultigrid levels as ex_compliance_multigrid.py:108-121 builds it.  With
        levels=None, coarsen while the grid halves evenly and the coarse level has > max_coarse_dofs.
        `coarse_smooth_steps` (default: smooth_steps) applies to every level below the finest; a list gives
        the levels below the finest their own values (the last entry repeats).
        smoother="chebyshev" replaces the damped-Jacobi sweeps by a Chebyshev smoother of degree
        smooth_steps (coarse_smooth_steps below the finest level) on [lmax/cheb_ratio, lmax].
        coarse_lag=True: the coarsest direct solve of an FP32 hierarchy keeps using the inverse of the previous
        update's coarse matrix until the current one is factorised (see DenseCholesky; MixedPrecisionCG
        switches to the new inverse between two iterations as soon as it exists)."""
        css = smooth_steps if coarse_smooth_steps is None else coarse_smooth_steps
        css_of = (lambda i: css[min(i, len(css) - 1)]) if isinstance(css, (list, tuple)) else (lambda i: css)
        if smoother not in ("jacobi", "chebyshev"):
            raise ValueError("smoother must be 'jacobi' or 'chebyshev'")

        def make(steps):
            if smoother == "chebyshev":
                return Chebyshev(degree=steps, ratio=cheb_ratio)
            return DampedJacobi(w=smoother_w)

        mgs = [cls(domain, smoother=make(smooth_steps), smooth_steps=smooth_steps, precision=precision)]
        while True:
            if levels is not None and len(mgs) >= levels - 1:
                break
            sub = mgs[-1].sub_domain
            g = Grid(*grid_of(sub))
            if levels is None and (not g.can_coarsen() or g.ndof <= max_coarse_dofs):
                break
            if not g.can_coarsen():
                raise ValueError(f"cannot build {levels} levels: grid {g.dims} does not halve evenly")
            steps = css_of(len(mgs) - 1)
            mgs.append(cls(sub, smoother=make(steps), smooth_steps=steps, precision=precision))
            mgs[-2].inner_level = mgs[-1]
        if coarse_lag:
            mgs[-1].inner_level = DenseCholesky(lag=True)
        return mgs


class _CaptureResult:
    def __init__(self):
        self.result = None
        self.launches = 0


def capture_graph(fn):
    """Capture fn() (device work on the current torch stream only, no host synchronisation) into a CUDA
    graph.  Returns (graph, info) with info.result = fn's return value and info.launches = kernels
    launched.  Every tensor fn allocates comes from the graph's private pool and is kept alive by the
    returned objects."""
    info = _CaptureResult()
    probe = _lib.Probe(targets=set())       # counts launches, records no events
    prev = _lib.Probe.active
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    try:
        _lib.Probe.active = probe
        with torch.cuda.graph(graph):
            info.result = fn()
    finally:
        _lib.Probe.active = prev
    info.launches = probe.launches
    return graph, info


def _check_coarsest(pc):
    """check() the coarsest direct solver below a multigrid chain (after its factorisation was queued)."""
    lv = pc
    while isinstance(lv, GeometricMultigrid):
        lv = lv.inner_level
    if isinstance(lv, DenseCholesky):
        lv.check()


def _side_stream(owner):
    """A second CUDA stream of `owner` (created once per device), for setup work that overlaps the main one.
    It has the higher priority: its kernels are small and on the critical path (the hierarchy the first
    preconditioner application waits for, the coarsest factorisation a lagged solve waits to promote), so
    the CTA scheduler should start them ahead of the bulk of the main stream's work."""
    dev = torch.cuda.current_device()
    s = getattr(owner, "_side", None)
    if s is None or s.device.index != dev:
        s = owner._side = torch.cuda.Stream(device=dev, priority=-1)
    return s


class _Scalars:
    """Device FP64 scalars of one CG instance: pq, pr, rr, qz, bb, zz."""

    def __init__(self, device):
        self.t = torch.zeros(8, dtype=torch.float64, device=device)

    def __getitem__(self, i):
        return self.t[i:i + 1]


def pcg(A, b, M, x, tol, maxit, restart, bnorm=None, callback=None):
    """Device PCG with the update formulas of pymoto/solvers/iterative.py:340-403 (x updated in place).

    Returns (iterations, final recursive relative residual).  `bnorm` overrides ||b|| in the stopping
    test (used by the mixed-precision refinement).
    """
    code = _lib.dtype_code(b)
    n = b.numel()
    ws = Workspace.get(b.device)
    sc = _Scalars(b.device)
    st = stream()
    r = A.apply(RESIDUAL, x, b)
    call("pmg_dot2", code, n, b, b, r, r, sc[4], ws.reduce, st)  # sc4 = b.b, sc5 = r.r
    bb, rr = sc.t[4:6].tolist()
    bn = math.sqrt(bb) if bnorm is None else bnorm
    if bn == 0.0:
        bn = 1.0
    res = math.sqrt(rr) / bn
    if res <= tol:
        return 0, res
    z = M(r)
    call("pmg_dot", code, n, z, z, sc[5], ws.reduce, st)
    p = torch.empty_like(b)
    call("pmg_scale_rsqrt", code, n, p, z, sc[5], st)
    q = torch.empty_like(b)
    it = 0
    for it in range(maxit):
        A.apply(MATVEC, p, out=q)
        call("pmg_dot2", code, n, p, q, p, r, sc[0], ws.reduce, st)  # pq, pr
        if it % restart == 0:
            call("pmg_axpy_ratio", code, n, x, p, sc[1], sc[0], 1.0, st)
            A.apply(RESIDUAL, x, b, out=r)
            call("pmg_dot", code, n, r, r, sc[2], ws.reduce, st)
        else:
            call("pmg_cg_update", code, n, x, r, p, q, sc[1], sc[0], sc[2], ws.reduce, st)
        res = math.sqrt(max(sc.t[2].item(), 0.0)) / bn
        if callback is not None:
            callback(it, res)
        if res <= tol or not math.isfinite(res):
            break
        z = M(r)
        call("pmg_dot", code, n, q, z, sc[3], ws.reduce, st)
        call("pmg_xpby_ratio", code, n, p, z, sc[3], sc[0], st)
    return it + 1, res


def pcg_fixed(A, b, M, x, k, bufs):
    """Exactly k PCG iterations from x = 0 with the update formulas of pcg(), without any host
    synchronisation (so it can be captured in a CUDA graph).  bufs = (r, p, q, scalars[8])."""
    code = _lib.dtype_code(b)
    n = b.numel()
    ws = Workspace.get(b.device)
    st = stream()
    r, p, q, sc = bufs
    x.zero_()
    r.copy_(b)
    z = M(r)
    call("pmg_dot", code, n, z, z, sc[5:6], ws.reduce, st)
    call("pmg_scale_rsqrt", code, n, p, z, sc[5:6], st)
    for i in range(k):
        A.apply(MATVEC, p, out=q)
        call("pmg_dot2", code, n, p, q, p, r, sc[0:1], ws.reduce, st)   # pq, pr
        call("pmg_cg_update", code, n, x, r, p, q, sc[1:2], sc[0:1], sc[2:3], ws.reduce, st)
        if i < k - 1:
            z = M(r)
            call("pmg_dot", code, n, q, z, sc[3:4], ws.reduce, st)
            call("pmg_xpby_ratio", code, n, p, z, sc[3:4], sc[0:1], st)
    return x


class CG(LinearSolver):
    """Preconditioned conjugate gradient (pymoto/solvers/iterative.py:295-403), on the device."""

    def __init__(self, A=None, preconditioner=None, tol=1e-7, maxit=10000, restart=50, verbosity=0):
        self.preconditioner = Preconditioner() if preconditioner is None else preconditioner
        self.A = A
        self.tol = tol
        self.maxit = maxit
        self.restart = restart
        self.verbosity = verbosity
        self.iterations = 0
        self.last_residual = None
        super().__init__(A)

    def update(self, A):
        t0 = time.perf_counter()
        if isinstance(A, StiffnessOperator):
            if getattr(self, "_Ap", None) is None or self._Ap.code != A.code or self._Ap.grid.dims != A.grid.dims:
                self._Ap = StiffnessOperator.like(A, A.code)
            A = self._Ap.assign(A, derived=False)
            # the preconditioner setup (Galerkin chain, coarsest factorisation) needs only the element scaling:
            # it runs on a side stream while the main stream reassembles the operator's stencil and diagonal
            main, side = torch.cuda.current_stream(), _side_stream(self)
            side.wait_stream(main)
            A.refresh_derived()
            with torch.cuda.stream(side):
                self.preconditioner.update(A)
            main.wait_stream(side)
        else:
            self.preconditioner.update(A)
        self.A = A
        if self.verbosity >= 1:
            torch.cuda.synchronize()
            print(f"CG Preconditioner set up in {np.round(time.perf_counter() - t0, 3)}s")

    def solve(self, rhs, x0=None, trans="N"):
        if trans not in ("N", "T", "H"):
            raise TypeError("Only N, T, or H transposition is possible")
        A = self.A
        b, kind = _to_device(rhs, A.torch_dtype)
        x = torch.zeros_like(b) if x0 is None else _to_device(x0, A.torch_dtype)[0].clone()
        t0 = time.perf_counter()
        it, res = pcg(A, b, self.preconditioner.solve, x, self.tol, self.maxit, self.restart)
        _check_coarsest(self.preconditioner)
        self.iterations, self.last_residual = it, res
        if not res <= self.tol:   # also a non-finite residual (NaN / Inf in the data)
            warnings.warn(f"CG Maximum iterations ({self.maxit}) reached, with final residuals {res}")
        elif self.verbosity >= 1:
            print(f"CG Converged in {it} iterations and {np.round(time.perf_counter() - t0, 3)}s, "
                  f"with final (max) residual {res}")
        return _from_device(x, kind)


class MixedPrecisionCG(LinearSolver):
    """Flexible CG in FP64 around an FP32 multigrid preconditioner.

    FP64: the solution, the residual, the operator products q = K(x) p, the alpha/beta dot products and the
    stopping test ||f - K(x) u|| / ||f|| <= tol (the recursive residual, recomputed explicitly every
    `restart` iterations and once more before returning).
    FP32: the preconditioner -- one V-cycle of the FP32 hierarchy (inner_iters=0) or exactly `inner_iters`
    FP32 PCG iterations on the FP32 operator (no host synchronisation: the whole preconditioner is one
    CUDA-graph replay, captured once per update()).
    Because the preconditioner is inexact (and may be nonlinear), directions are K-orthogonalised against
    the last `m` directions (FCG(m)); the reference's beta = -(q.z)/(p.q) is the m = 1 case.
    `warm_start` is an optional learned predictor (pymoto_gb300.learned.LearnedWarmStart): its prediction and
    the given x0 span the space in which the initial guess is the energy-optimal (Rayleigh-Ritz)
    combination (Gram products on the FP32 operator, one FP64 residual), every converged solution is passed
    back to it for training, and with its `coarse_correction` the prediction also deflates every
    preconditioner application (A-DEF2); `coarse_correction` here is an optional callable r64 -> z64 added to
    the preconditioned residual.  With a lagged coarsest solve (DenseCholesky(lag=True)) the new coarse
    inverse is promoted between two iterations as soon as its factorisation has finished.
    """

    def __init__(self, A=None, preconditioner=None, tol=1e-6, m=2, inner_iters=0, inner_tol=0.1, maxit=500,
                 restart=50, verbosity=0, warm_start=None, coarse_correction=None, fallback=True, stall_window=30,
                 verify_residual=True):
        """verify_residual: recompute ||f - K u|| explicitly in FP64 once the recursive residual is below tol
        (and continue if it is not); False stops on the recursive residual like the reference CG
        (pymoto/solvers/iterative.py:386-390)."""
        self.verify_residual = verify_residual
        self.preconditioner = preconditioner
        self.fallback = fallback
        self.stall_window = stall_window
        self.fell_back = False
        self._fallback_pc = None
        self.tol = tol
        self.m = max(1, int(m))
        self.inner_iters = inner_iters
        self.inner_tol = inner_tol
        self.maxit = maxit
        self.restart = restart
        self.verbosity = verbosity
        self.warm_start = warm_start
        self.warm_start_active = True      # False during adjoint solves (set by LinSolve)
        self.coarse_correction = coarse_correction
        self.iterations = 0
        self.inner_iterations = 0
        self.last_residual = None
        super().__init__(A)

    def update(self, A):
        if self.warm_start is not None and isinstance(A, ScalarOperator):
            raise NotImplementedError("the learned warm start predicts displacement fields (3 components per node)")
        if getattr(self, "_A64", None) is None or type(self._A64) is not type(A) or self._A64.grid.dims != A.grid.dims:
            self._A64 = type(A).like(A, F64)
        # the FP32 hierarchy is built from the element scaling of A alone: on a side stream, overlapping the
        # FP64 stencil assembly of the outer operator on the main stream
        main, side = torch.cuda.current_stream(), _side_stream(self)
        side.wait_stream(main)
        self.A64 = self._A64.assign(A)
        self.A = self.A64
        with torch.cuda.stream(side):
            if self.preconditioner is not None:
                self.preconditioner.update(A)
                lv0 = getattr(self.preconditioner, "A", None)
                self.A32 = lv0 if type(lv0) is type(A) and lv0.code == F32 else A.astype(F32)
            else:
                self.A32 = A.astype(F32)
        # joined just before the first preconditioner application of the next solve, so the FP64 work that
        # precedes it (initial residual, warm-start products) also overlaps the hierarchy set-up; with a lagged
        # coarsest solve only up to the event that marks the hierarchy ready (its factorisation keeps running)
        lv = self.preconditioner
        while isinstance(lv, GeometricMultigrid):
            lv = lv.inner_level
        ev = getattr(lv, "ready_event", None) if isinstance(lv, DenseCholesky) and lv.lag else None
        self._side_pending = ev if ev is not None else side
        self._lagged_coarse = lv if ev is not None else None
        self._fallback_ready = False
        n, dev = self.A64.shape[0], self.A64.device
        if getattr(self, "_r32", None) is None or self._r32.numel() != n or self._r32.device != dev:
            f32 = dict(dtype=torch.float32, device=dev)
            self._r32 = torch.empty(n, **f32)
            self._z32 = torch.empty(n, **f32)
            self._inner_bufs = (torch.empty(n, **f32), torch.empty(n, **f32), torch.empty(n, **f32),
                                torch.zeros(8, dtype=torch.float64, device=dev))
            self._inner_graph = None

    def _inner(self):
        """k fixed FP32 PCG iterations on self._r32 -> self._z32, as a CUDA graph captured per update."""
        run = lambda: pcg_fixed(self.A32, self._r32, self.preconditioner.solve, self._z32, self.inner_iters,
                                self._inner_bufs)
        if self._inner_graph is None:
            run()                                     # eager run: loads every kernel before the capture
            self._inner_graph, info = capture_graph(run)
            self._inner_launches = info.launches
        _lib.replay(f"inner_pcg{self.inner_iters}", self._inner_graph, self._inner_launches)
        self.inner_iterations += self.inner_iters
        return self._z32

    def _fp64_preconditioner(self):
        """The same multigrid hierarchy in FP64: the fallback when the FP32 preconditioner stalls."""
        if self._fallback_pc is None:
            chain, lv = [], self.preconditioner
            while isinstance(lv, GeometricMultigrid):
                sm = lv.smoother
                chain.append(GeometricMultigrid(lv.domain, smoother=DampedJacobi(w=getattr(sm, "w", 0.5)),
                                                smooth_steps=lv.smooth_steps, precision="fp64"))
                if len(chain) > 1:
                    chain[-2].inner_level = chain[-1]
                lv = lv.inner_level
            self._fallback_pc = chain[0] if chain else DampedJacobi(w=1.0)
        if not self._fallback_ready:
            self._fallback_pc.update(self.A64)   # shares the persistent FP64 operator
            self._fallback_ready = True
        return self._fallback_pc

    def _precondition(self, r, rn, z):
        """z (FP64) = ||r|| M32(r / ||r||), or the FP64 fallback preconditioner once switched."""
        n = r.numel()
        st = stream()
        if self.fell_back:
            z.copy_(self._fp64_preconditioner().solve(r))
            return z
        call("pmg_convert", F64, F32, n, r, self._r32, 1.0 / rn, st)
        if self.preconditioner is None:
            z32 = self._r32
        elif self.inner_iters > 0:
            z32 = self._inner()
        else:
            z32 = self.preconditioner.solve(self._r32)
        call("pmg_convert", F32, F64, n, z32, z, rn, st)
        if self.coarse_correction is not None:
            z.add_(self.coarse_correction(r))
        return z

    # ---------------------------------------------------------------------------------- FCG iteration
    def _ensure_fcg_buffers(self, n, dev):
        k = self.m + 1
        bufs = getattr(self, "_fcg", None)
        if bufs is not None and bufs["n"] == n and bufs["dev"] == dev and bufs["k"] == k:
            return bufs
        f64 = dict(dtype=torch.float64, device=dev)
        bufs = {"n": n, "dev": dev, "k": k, "x": torch.empty(n, **f64), "b": torch.empty(n, **f64),
                "r": torch.empty(n, **f64), "z": torch.empty(n, **f64),
                "P": [torch.zeros(n, **f64) for _ in range(k)], "Q": [torch.zeros(n, **f64) for _ in range(k)],
                # scalars: 0 bb, 1 rr, 2 pr, 3.. 3+k q_j.z, 3+k.. 3+2k p_j.q_j
                "s": torch.zeros(3 + 2 * k, **f64), "graphs": [None] * k, "seen": [False] * k}
        self._fcg = bufs
        return bufs

    def _fcg_step(self, slot):
        """One FCG(m) iteration writing its direction into history slot `slot` (device work only)."""
        B = self._fcg
        A, n, k = self.A64, B["n"], B["k"]
        s, P, Q = B["s"], B["P"], B["Q"]
        ws = Workspace.get(B["dev"])
        st = stream()
        r, z, x = B["r"], B["z"], B["x"]
        lc = B.get("learned_cc")
        rin = r
        if lc is not None:
            # deflation on the span of the network's prediction w (A-DEF2): the preconditioner sees
            # r - (w.r / w.Kw) Kw, and (w.r / w.Kw) w is added to its output; no-ops while w.Kw = 0
            w, kw, rdef, num, den = lc
            call("pmg_dot", F64, n, w, r, num, ws.reduce, st)
            rdef.copy_(r)
            call("pmg_axpy_ratio", F64, n, rdef, kw, num, den, -1.0, st)
            rin = rdef
        if self.fell_back:
            z.copy_(self._fp64_preconditioner().solve(rin))
        else:
            call("pmg_convert_dscale", F64, F32, n, rin, self._r32, s[1:2], 1, st)
            if self.preconditioner is None:
                z32 = self._r32
            elif self.inner_iters > 0:
                z32 = pcg_fixed(self.A32, self._r32, self.preconditioner.solve, self._z32, self.inner_iters,
                                self._inner_bufs)
            else:
                z32 = self.preconditioner.solve(self._r32)
            call("pmg_convert_dscale", F32, F64, n, z32, z, s[1:2], 0, st)
        if self.coarse_correction is not None:
            z.add_(self.coarse_correction(r))
        if lc is not None:
            call("pmg_axpy_ratio", F64, n, z, w, num, den, 1.0, st)
        p, q = P[slot], Q[slot]
        p.copy_(z)
        for j in range(k):           # K-orthogonalise against the other (older) directions
            if j == slot:
                continue
            call("pmg_dot", F64, n, Q[j], z, s[3 + j:4 + j], ws.reduce, st)
            call("pmg_axpy_ratio", F64, n, p, P[j], s[3 + j:4 + j], s[3 + k + j:4 + k + j], -1.0, st)
        A.apply(MATVEC, p, out=q)
        pq = s[3 + k + slot:4 + k + slot]
        call("pmg_dot2", F64, n, p, q, p, r, self._pqpr, ws.reduce, st)
        pq.copy_(self._pqpr[0:1])
        s[2:3].copy_(self._pqpr[1:2])
        call("pmg_cg_update", F64, n, x, r, p, q, s[2:3], pq, s[1:2], ws.reduce, st)

    def _set_learned_correction(self, A, B, vecs, n, dev):
        """Coarse space of the learned warm start (`coarse_correction=True` on it): the masked prediction w of
        this solve, Kw and w.Kw, or w.Kw = 0 (deflation off) when no prediction was used.  The buffers keep
        their addresses, so the captured FCG step stays valid."""
        ws_ = self.warm_start
        if ws_ is None or not getattr(ws_, "coarse_correction", False):
            return
        if B.get("learned_cc") is None:
            f64 = dict(dtype=torch.float64, device=dev)
            B["learned_cc"] = (torch.zeros(n, **f64), torch.zeros(n, **f64), torch.zeros(n, **f64),
                               torch.zeros(1, **f64), torch.zeros(1, **f64))
            for j in range(B["k"]):              # graphs captured without the correction: recapture
                B["graphs"][j] = None
        w, kw, _, _, den = B["learned_cc"]
        if getattr(ws_, "_predicted", False) and vecs:
            st = stream()
            w.copy_(vecs[-1])                    # the masked prediction (last Rayleigh-Ritz direction)
            A.apply(MATVEC, w, out=kw)
            call("pmg_dot", F64, n, w, kw, den, Workspace.get(dev).reduce, st)
        else:
            den.zero_()

    def _join_setup(self):
        side = getattr(self, "_side_pending", None)
        if side is not None:
            if isinstance(side, torch.cuda.Event):
                torch.cuda.current_stream().wait_event(side)
            else:
                torch.cuda.current_stream().wait_stream(side)
            self._side_pending = None

    def _run_step(self, slot):
        self._join_setup()
        B = self._fcg
        if self.fell_back or not self.use_graph:
            self._fcg_step(slot)
            return
        g = B["graphs"][slot]
        if g is None:
            if not B["seen"][slot]:            # first use of this slot: eager (loads every kernel)
                B["seen"][slot] = True
                self._fcg_step(slot)
                return
            B["graphs"][slot], info = capture_graph(lambda: self._fcg_step(slot))
            B.setdefault("launches", {})[slot] = info.launches
            self._fcg_step_replay(slot)
            return
        self._fcg_step_replay(slot)

    def _fcg_step_replay(self, slot):
        B = self._fcg
        _lib.replay(f"fcg_step|m={self.m}|inner={self.inner_iters}", B["graphs"][slot], B["launches"][slot])
        if self.inner_iters > 0:
            self.inner_iterations += self.inner_iters

    use_graph = True

    def solve(self, rhs, x0=None, trans="N"):
        A = self.A64
        b_in, kind = _to_device(rhs, torch.float64)
        n = b_in.numel()
        dev = b_in.device
        B = self._ensure_fcg_buffers(n, dev)
        if getattr(self, "_pqpr", None) is None or self._pqpr.device != dev:
            self._pqpr = torch.zeros(2, dtype=torch.float64, device=dev)
        x, b, r = B["x"], B["b"], B["r"]
        b.copy_(b_in)
        ws = Workspace.get(dev)
        st = stream()
        s = B["s"]
        # the learned warm start predicts the response to the load of the design, not to other right-hand sides:
        # LinSolve switches it off (warm_start_active) for the adjoint solves of the sensitivities
        learn = self.warm_start is not None and trans == "N" and getattr(self, "warm_start_active", True)
        extra = self.warm_start.basis(A, x0) if learn else []
        if extra:
            # initial guess: energy-optimal combination of the given guess, older solutions and the network's
            # prediction (all with their constrained dofs zeroed)
            from .learned import rayleigh_ritz
            k = len(extra) + (x0 is not None)
            if len(B.get("wsv", [])) < len(extra):
                B["wsv"] = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(len(extra))]
            if len(B.get("wsq", [])) < k:
                B["wsq"] = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(k)]
            vecs = [] if x0 is None else [_to_device(x0, torch.float64)[0].contiguous()]
            for v, buf in zip(extra, B["wsv"]):
                call("pmg_mask_bc", F64, getattr(A, "ncomp", A.grid.dim), A.grid.nnodes, A.bcmask, 0, v, buf, st)
                vecs.append(buf)
            # Gram products on the FP32 level-0 operator of the hierarchy once the set-up stream has it
            pc = self.preconditioner
            ev = getattr(pc, "level0_ready", None)
            a32 = getattr(self, "A32", None)
            if ev is not None and a32 is not None and a32 is getattr(pc, "A", None) and a32.shape[0] == n:
                torch.cuda.current_stream().wait_event(ev)
                self.warm_start_coefficients = rayleigh_ritz(A, b, vecs, x, r, B["wsq"], A32=a32,
                                                             work32=(self._r32, self._z32))
            else:
                self.warm_start_coefficients = rayleigh_ritz(A, b, vecs, x, r, B["wsq"])
            if hasattr(self.warm_start, "report"):
                self.warm_start.report(getattr(rayleigh_ritz, "last_shares", []))
        else:
            vecs = []
            if x0 is not None:
                x.copy_(_to_device(x0, torch.float64)[0])
            else:
                x.zero_()
            A.apply(RESIDUAL, x, b, out=r)
        if learn:
            self._set_learned_correction(A, B, vecs, n, dev)
        call("pmg_dot2", F64, n, b, b, r, r, s[0:1], ws.reduce, st)
        bb, rr = s[0:2].tolist()
        bn = math.sqrt(bb) or 1.0
        res = math.sqrt(max(rr, 0.0)) / bn
        self.inner_iterations = 0
        self.fell_back = False
        can_fall_back = self.fallback and self.preconditioner is not None
        it, it_fb, best, best_it = 0, 0, res, 0
        while res > self.tol:
            # fresh direction history (slots zeroed: zero products give zero projections)
            for t in B["P"] + B["Q"]:
                t.zero_()
            s[3:].zero_()
            slot = 0
            while res > self.tol:
                if can_fall_back and not self.fell_back and (it >= self.maxit or it - best_it >= self.stall_window):
                    self.fell_back = True          # FP32 preconditioning stalled: FP64 hierarchy from here on
                    it_fb = it
                    for t in B["P"] + B["Q"]:
                        t.zero_()
                    s[3:].zero_()
                    slot = 0
                    if self.verbosity >= 1:
                        print(f"MixedPrecisionCG: FP32 preconditioner stalled at {res:.3e}; FP64 fallback")
                if (self.fell_back or not can_fall_back) and it - it_fb >= self.maxit:
                    break
                self._run_step(slot)
                slot = (slot + 1) % B["k"]
                it += 1
                res = math.sqrt(max(s[1].item(), 0.0)) / bn
                if getattr(self, "_lagged_coarse", None) is not None and self._lagged_coarse.promote_if_ready():
                    self._lagged_coarse = None    # the exact coarse solve of this update from the next step on
                if self.verbosity >= 2:
                    print(f"FCG it {it}: residual {res:.3e}")
                if res < 0.5 * best:
                    best, best_it = res, it
                if not math.isfinite(res):
                    break
            if not self.verify_residual:
                break
            # true FP64 residual; continue from it if the recursive residual drifted
            A.apply(RESIDUAL, x, b, out=r)
            call("pmg_dot", F64, n, r, r, s[1:2], ws.reduce, st)
            res = math.sqrt(max(s[1].item(), 0.0)) / bn
            if not math.isfinite(res) or ((self.fell_back or not can_fall_back) and it - it_fb >= self.maxit):
                break
        self._join_setup()
        if self.preconditioner is not None:
            _check_coarsest(self.preconditioner)
        self.iterations, self.last_residual = it, res
        # the explicit FP64 residual b - A x of the returned solution (LinSolve derives A x from it)
        self.final_residual = r if trans == "N" else None
        if learn and math.isfinite(res):
            self.warm_start.observe(A, x)
        if not res <= self.tol:   # also a non-finite residual (NaN / Inf in the data)
            warnings.warn(f"MixedPrecisionCG did not reach tol {self.tol}: residual {res}")
        out = x.clone()
        return _from_device(out, kind)


def default_solver(A, tol=1e-10):
    """CG with an automatically sized FP64 multigrid hierarchy (used when LinSolve gets no solver)."""
    from .domain import VoxelDomain
    g = A.grid
    if g.can_coarsen():
        mgs = GeometricMultigrid.hierarchy(VoxelDomain(*g.dims), smoother_w=0.5, smooth_steps=2)
        return CG(preconditioner=mgs[0], tol=tol, maxit=5000)
    return CG(preconditioner=DampedJacobi(w=1.0), tol=tol, maxit=20000)
