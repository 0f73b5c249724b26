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
from .operators import TORCH_DTYPE, Grid, StencilOperator, StiffnessOperator, Workspace

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
        rn, bn = out.sqrt().tolist()
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


class DenseCholesky(LinearSolver):
    """Direct solve of the coarsest Galerkin operator: dense FP64 banded Cholesky on the device.

    Stands in for SolverSparseLU (pymoto/solvers/sparse.py:515-555), which auto_determine_solver picks for
    the coarse sparse matrix (pymoto/solvers/auto_determine.py:109-122).  The factorisation is FP64; an
    FP32 copy of the factor serves FP32 right-hand sides.
    """

    MAX_DOFS = 20000

    def __init__(self, A=None):
        self.L = None
        self.L32 = None
        super().__init__(A)

    def update(self, A):
        if not isinstance(A, StencilOperator):
            raise TypeError("DenseCholesky expects a coarse StencilOperator")
        n = A.grid.ndof
        if n > self.MAX_DOFS:
            raise ValueError(f"coarsest level has {n} dofs (> {self.MAX_DOFS}); add multigrid levels")
        self.n = n
        self.bw = A.bandwidth()
        L = A.to_dense()
        info = torch.zeros(1, dtype=torch.int32, device=L.device)
        call("pmg_cholesky_factor", n, L, self.bw, info, stream())
        bad = int(info.item())
        if bad != 0:
            raise np.linalg.LinAlgError(f"coarsest-level matrix not positive definite (pivot {bad - 1})")
        self.L = L
        self.L32 = L.to(torch.float32) if A.code == F32 else None

    def solve(self, rhs, x0=None, trans="N"):
        code = _lib.dtype_code(rhs)
        L = self.L if code == F64 else self.L32
        if L is None:
            L = self.L32 = self.L.to(torch.float32)
        out = torch.empty_like(rhs)
        call("pmg_cholesky_solve", code, self.n, L, self.bw, rhs.contiguous(), out, stream())
        return out


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
        super().__init__(A)

    def update(self, A):
        code = self.precision if self.precision is not None else A.code
        op = A.astype(code) if isinstance(A, StiffnessOperator) else A
        if op.code != code:
            raise TypeError("coarse operators keep the precision of their parent level")
        self.A = op
        self.smoother.update(op)
        Ac = op.galerkin()
        if self.inner_level is None:
            self.inner_level = DenseCholesky()
        if isinstance(self.inner_level, GeometricMultigrid) and self.inner_level.precision is None:
            self.inner_level.precision = code
        self.inner_level.update(Ac)
        n = self.grid.ndof
        if self._buf is None or self._buf[0].dtype != op.torch_dtype or self._buf[0].device != op.device:
            self._buf = [torch.empty(n, dtype=op.torch_dtype, device=op.device) for _ in range(3)]

    @property
    def code(self):
        return self.A.code

    def solve(self, rhs, x0=None, trans="N"):
        in_code = _lib.dtype_code(rhs)
        b = rhs if in_code == self.A.code else rhs.to(self.A.torch_dtype)
        u = self._vcycle(b, x0 if x0 is None or x0.dtype == b.dtype else x0.to(b.dtype))
        return u if in_code == self.A.code else u.to(rhs.dtype)

    def _vcycle(self, b, x0=None):
        A, w, steps = self.A, None, self.smooth_steps
        u, t, r = self._buf
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
        rc = torch.empty(g.coarse().ndof, dtype=b.dtype, device=b.device)
        call("pmg_restrict", A.code, g.nelx, g.nely, g.nelz, r, rc, stream())
        uc = inner._vcycle(rc) if isinstance(inner, GeometricMultigrid) else inner.solve(rc)
        call("pmg_prolong_add", A.code, g.nelx, g.nely, g.nelz, uc, u, stream())
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

    @classmethod
    def hierarchy(cls, domain, levels=None, smoother_w=0.5, smooth_steps=5, precision=None, max_coarse_dofs=3000):
        """Chain of GeometricMultigrid levels as ex_compliance_multigrid.py:108-121 builds it.  With
        levels=None, coarsen while the grid halves evenly and the coarse level has > max_coarse_dofs."""
        mgs = [cls(domain, smoother=DampedJacobi(w=smoother_w), smooth_steps=smooth_steps, precision=precision)]
        while True:
            if levels is not None and len(mgs) >= levels - 1:
                break
            sub = mgs[-1].sub_domain
            g = Grid(*grid_of(sub))
            if levels is None and (not g.can_coarsen() or g.ndof <= max_coarse_dofs):
                break
            if not g.can_coarsen():
                raise ValueError(f"cannot build {levels} levels: grid {g.dims} does not halve evenly")
            mgs.append(cls(sub, smoother=DampedJacobi(w=smoother_w), smooth_steps=smooth_steps, precision=precision))
            mgs[-2].inner_level = mgs[-1]
        return mgs


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
        self.A = A
        self.preconditioner.update(A)
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
        self.iterations, self.last_residual = it, res
        if res > self.tol:
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
    FP32: the preconditioner -- one V-cycle of the FP32 hierarchy (inner_iters=0) or up to `inner_iters`
    FP32 PCG iterations on the FP32 operator to the relative tolerance `inner_tol`.
    Because the preconditioner is inexact (and may be nonlinear), directions are K-orthogonalised against
    the last `m` directions (FCG(m)); the reference's beta = -(q.z)/(p.q) is the m = 1 case.
    `warm_start` is an optional object with `.predict(A, rhs)` giving the initial guess when no x0 is
    passed; `coarse_correction` an optional callable r64 -> z64 added to the preconditioned residual.
    """

    def __init__(self, A=None, preconditioner=None, tol=1e-6, m=4, inner_iters=0, inner_tol=0.1, maxit=500,
                 restart=50, verbosity=0, warm_start=None, coarse_correction=None):
        self.preconditioner = preconditioner
        self.tol = tol
        self.m = max(1, int(m))
        self.inner_iters = inner_iters
        self.inner_tol = inner_tol
        self.maxit = maxit
        self.restart = restart
        self.verbosity = verbosity
        self.warm_start = warm_start
        self.coarse_correction = coarse_correction
        self.iterations = 0
        self.inner_iterations = 0
        self.last_residual = None
        super().__init__(A)

    def update(self, A):
        self.A64 = A.astype(F64)
        self.A32 = A.astype(F32)
        self.A = self.A64
        if self.preconditioner is not None:
            self.preconditioner.update(self.A32)

    def _precondition(self, r, rn, z):
        """z (FP64) = ||r|| M32(r / ||r||)."""
        n = r.numel()
        st = stream()
        call("pmg_convert", F64, F32, n, r, self._r32, 1.0 / rn, st)
        if self.preconditioner is None:
            z32 = self._r32
        elif self.inner_iters > 0:
            z32 = self._z32
            z32.zero_()
            its, _ = pcg(self.A32, self._r32, self.preconditioner.solve, z32, self.inner_tol, self.inner_iters,
                         self.restart)
            self.inner_iterations += its
        else:
            z32 = self.preconditioner.solve(self._r32)
        call("pmg_convert", F32, F64, n, z32, z, rn, st)
        if self.coarse_correction is not None:
            z.add_(self.coarse_correction(r))
        return z

    def solve(self, rhs, x0=None, trans="N"):
        A = self.A64
        b, kind = _to_device(rhs, torch.float64)
        n = b.numel()
        dev = b.device
        if x0 is not None:
            x = _to_device(x0, torch.float64)[0].clone()
        elif self.warm_start is not None:
            x = self.warm_start.predict(A, b).to(torch.float64).contiguous()
        else:
            x = torch.zeros_like(b)
        ws = Workspace.get(dev)
        st = stream()
        self._r32 = torch.empty(n, dtype=torch.float32, device=dev)
        self._z32 = torch.empty(n, dtype=torch.float32, device=dev)
        sc = torch.zeros(2 + self.m, dtype=torch.float64, device=dev)   # bb | rr, q_j.z ...
        r = A.apply(RESIDUAL, x, b)
        call("pmg_dot2", F64, n, b, b, r, r, sc[0:1], ws.reduce, st)
        bb, rr = sc[0:2].tolist()
        bn = math.sqrt(bb) or 1.0
        res = math.sqrt(rr) / bn
        self.inner_iterations = 0
        it = 0
        hist = []               # FIFO of the last m (p, K p, [p.Kp, p.r]) triples
        z = torch.empty_like(b)
        while res > self.tol and it < self.maxit:
            self._precondition(r, res * bn, z)
            # p = z - sum_j (q_j.z)/(p_j.q_j) p_j
            p = z.clone()
            for j, (pj, qj, sj) in enumerate(hist):
                call("pmg_dot", F64, n, qj, z, sc[2 + j:3 + j], ws.reduce, st)
                call("pmg_axpy_ratio", F64, n, p, pj, sc[2 + j:3 + j], sj[0:1], -1.0, st)
            q = A.apply(MATVEC, p, out=hist[0][1] if len(hist) == self.m else None)
            s2 = torch.empty(2, dtype=torch.float64, device=dev)
            call("pmg_dot2", F64, n, p, q, p, r, s2, ws.reduce, st)           # p.q, p.r
            it += 1
            if it % self.restart == 0:
                call("pmg_axpy_ratio", F64, n, x, p, s2[1:2], s2[0:1], 1.0, st)
                A.apply(RESIDUAL, x, b, out=r)
                call("pmg_dot", F64, n, r, r, sc[1:2], ws.reduce, st)
            else:
                call("pmg_cg_update", F64, n, x, r, p, q, s2[1:2], s2[0:1], sc[1:2], ws.reduce, st)
            res = math.sqrt(max(sc[1].item(), 0.0)) / bn
            if self.verbosity >= 2:
                print(f"FCG it {it}: residual {res:.3e}")
            if len(hist) == self.m:
                hist.pop(0)
            hist.append((p, q, s2))
            if not math.isfinite(res):
                break
        # final true FP64 residual
        A.apply(RESIDUAL, x, b, out=r)
        call("pmg_dot", F64, n, r, r, sc[1:2], ws.reduce, st)
        res = math.sqrt(max(sc[1].item(), 0.0)) / bn
        self.iterations, self.last_residual = it, res
        if res > self.tol:
            warnings.warn(f"MixedPrecisionCG did not reach tol {self.tol}: residual {res}")
        return _from_device(x, kind)


def default_solver(A, tol=1e-10):
    """CG with an automatically sized FP64 multigrid hierarchy (used when LinSolve gets no solver)."""
    from .domain import VoxelDomain
    g = A.grid
    if g.can_coarsen():
        mgs = GeometricMultigrid.hierarchy(VoxelDomain(*g.dims), smoother_w=0.5, smooth_steps=2)
        return CG(preconditioner=mgs[0], tol=tol, maxit=5000)
    return CG(preconditioner=DampedJacobi(w=1.0), tol=tol, maxit=20000)
