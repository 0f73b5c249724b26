"""CPU design iteration of the reference path, for the timed CPU baseline (test infrastructure only).

Restates how pyMOTO runs one design iteration of the multigrid compliance example
(examples/topology_optimization/ex_compliance_multigrid.py:81-162):
  * AssembleStiffness with reuse_sparsity: CSR pattern and data map built once, then every iteration
    data = 0; np.add.at(data, datamap, x (x) K0); data[bc diagonal] = bcdiagval
    (pymoto/modules/assembly.py:116-243, :245-296);
  * GeometricMultigrid.update: R built once, Ac = R^T A R per level, SuperLU on the coarsest level
    (pymoto/solvers/iterative.py:168-220);
  * LinSolve + LDAWrapper + CG to the relative tolerance (pymoto/modules/linalg.py:164-219,
    pymoto/solvers/solvers.py:140-306, pymoto/solvers/iterative.py:340-403);
  * FilterConv, SIMP, compliance, DyadicMatrix contraction, filter transpose and the OC update.
"""
import numpy as np
import scipy.sparse as sps

from .pymoto_oracle import (Grid, LinSolveOracle, MGLevel, cg_solve, conv_filter, conv_filter_T,
                            conv_filter_weights, default_bcdiagval, element_stiffness, oc_step, prolongation,
                            relative_residual, sensitivity_contract, simp, simp_derivative, vcycle)
from scipy.sparse.linalg import splu

__all__ = ["StructuredCSR", "CachedHierarchy", "ReferenceDesignLoop", "cantilever_loads", "fp64_cg_reference"]


class StructuredCSR:
    """CSR pattern + data map of K = sum_e x_e K0 on a voxel grid (pyMOTO's reuse_sparsity assembly)."""

    def __init__(self, grid, K0, bc=None, bcdiagval=None, chunk=65536):
        self.grid, self.K0 = grid, K0
        g = grid
        dim = g.dim
        nnx, nny, nnz = g.nelx + 1, g.nely + 1, g.nelz + 1
        koff = [-1, 0, 1] if dim == 3 else [0]
        offs = [(dx, dy, dz) for dz in koff for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
        nodes = np.arange(g.nnodes)
        ni, nj, nk = nodes % nnx, (nodes // nnx) % nny, nodes // (nnx * nny)
        valid = np.stack([(ni + dx >= 0) & (ni + dx < nnx) & (nj + dy >= 0) & (nj + dy < nny) & (nk + dz >= 0) &
                          (nk + dz < nnz) for dx, dy, dz in offs], axis=1)
        rank = np.cumsum(valid, axis=1) - valid                        # position of offset o among valid ones
        nvalid = valid.sum(axis=1)
        row_len = np.repeat(nvalid * dim, dim)
        self.indptr = np.zeros(g.ndof + 1, dtype=np.int64)
        np.cumsum(row_len, out=self.indptr[1:])
        nbr = nodes[:, None] + np.array([dx + nnx * (dy + nny * dz) for dx, dy, dz in offs])[None, :]
        cols_node = np.where(valid, nbr, -1)
        ind = (cols_node[:, :, None] * dim + np.arange(dim)).reshape(g.nnodes, -1)        # (nnodes, noff*dim)
        okmask = np.repeat(valid, dim, axis=1)
        per_row = ind[okmask.reshape(g.nnodes, -1)].reshape(-1)                           # row-major per node
        # every dof of a node has the same column list
        counts = nvalid * dim
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        self.indices = np.empty(self.indptr[-1], dtype=np.int64)
        for d in range(dim):
            # rows node*dim + d: copy the node's column list
            dst = self.indptr[nodes * dim + d]
            idx = np.repeat(dst - starts, counts) + np.arange(per_row.size)
            self.indices[idx] = per_row
        # data map (nel, nde, nde)
        nn = g.elemnodes
        nde = nn * dim
        loc = np.array([[a & 1, (a >> 1) & 1, (a >> 2) & 1] for a in range(nn)])
        oidx = {o: t for t, o in enumerate(offs)}
        otab = np.array([[oidx[tuple(int(v) for v in (loc[b] - loc[a]) * ([1, 1, 1] if dim == 3 else [1, 1, 0]))]
                          for b in range(nn)] for a in range(nn)])                       # (nn, nn)
        conn = g.conn()
        self.datamap = np.empty((g.nel, nde, nde), dtype=np.int64)
        cvec = np.arange(dim)
        for s in range(0, g.nel, chunk):
            c = conn[s:s + chunk]                                                         # (m, nn)
            rowstart = self.indptr[(c[:, :, None] * dim + cvec).reshape(c.shape[0], -1)]  # (m, nde)
            rk = rank[c[:, :, None], otab[None, :, :]]                                    # (m, nn, nn)
            rk = np.repeat(np.repeat(rk, dim, axis=1), dim, axis=2) * dim + np.tile(cvec, nn)[None, None, :]
            self.datamap[s:s + chunk] = rowstart[:, :, None] + rk
        self.datamap = self.datamap.reshape(-1)
        self.bc = None
        if bc is not None and len(bc):
            self.bc = np.asarray(bc, dtype=np.int64).ravel()
            self.bcdiagval = default_bcdiagval(K0) if bcdiagval is None else bcdiagval
            isbc = np.zeros(g.ndof, dtype=bool)
            isbc[self.bc] = True
            row_of = np.repeat(np.arange(g.ndof), np.diff(self.indptr))
            dc = g.dofconn()
            hit = (isbc[dc][:, :, None] | isbc[dc][:, None, :]).reshape(-1)
            # positions of the bc diagonal entries
            rs = self.indptr[self.bc]
            re = self.indptr[self.bc + 1]
            self.bcadd = np.array([rs[t] + np.searchsorted(self.indices[rs[t]:re[t]], self.bc[t]) for t in
                                   range(self.bc.size)], dtype=np.int64)
            self.datamap[hit] = self.bcadd[0]
            del row_of

    def assemble(self, x):
        scaled = (self.K0.reshape(1, -1) * x.reshape(-1, 1)).reshape(-1)
        data = np.zeros(self.indices.size)
        np.add.at(data, self.datamap, scaled)
        if self.bc is not None:
            data[self.bcadd] = self.bcdiagval
        n = self.grid.ndof
        return sps.csr_matrix((data, self.indices, self.indptr), shape=(n, n))


class CachedHierarchy:
    """GeometricMultigrid chain whose prolongations are built once (iterative.py:168-176)."""

    def __init__(self, grid, levels, w, smooth_steps):
        self.grids = [grid]
        for _ in range(levels - 1):
            self.grids.append(self.grids[-1].coarse())
        self.R = [prolongation(gr) for gr in self.grids[:-1]]
        self.w, self.smooth_steps = w, smooth_steps

    def update(self, A):
        lvls = []
        M = A
        for gr, R in zip(self.grids[:-1], self.R):
            lv = MGLevel.__new__(MGLevel)
            lv.grid, lv.A, lv.w, lv.smooth_steps = gr, M, self.w, self.smooth_steps
            lv.D = M.diagonal()
            lv.R = R
            lv.Ac = (R.T @ M @ R).tocsr()
            lv.inner, lv.lu = None, None
            if lvls:
                lvls[-1].inner = lv
            lvls.append(lv)
            M = lv.Ac
        lvls[-1].lu = splu(lvls[-1].Ac.tocsc())
        return lvls


class ReferenceDesignLoop:
    """One design iteration of the reference multigrid compliance example on a 3D/2D cantilever."""

    def __init__(self, shape, radius=2.5, levels=4, w=0.6, smooth_steps=2, tol=1e-6, move=0.2, seed=0,
                 volfrac=None):
        self.grid = g = Grid(*shape)
        nodes = g.nodes_where(i=0)
        self.bc = (nodes[:, None] * g.dim + np.arange(g.dim)).ravel()
        self.f = np.zeros(g.ndof)
        tip = g.node_number(g.nelx, g.nely // 2, g.nelz // 2)
        self.f[g.dim * tip + 1] = -1.0
        self.K0 = element_stiffness(g)
        self.W = conv_filter_weights(g, radius)
        self.csr = StructuredCSR(g, self.K0, self.bc)
        self.hier = CachedHierarchy(g, levels, w, smooth_steps)
        self.solver = LinSolveOracle(g, levels, w, smooth_steps, tol)
        self.solver.lda_tol = 5 * tol
        self._patch_solver()
        rng = np.random.default_rng(seed)
        self.x = rng.uniform(1e-3, 1.0, g.nel)
        self.volfrac = float(np.mean(self.x)) if volfrac is None else volfrac
        self.move = move

    def _patch_solver(self):
        hier, solver = self.hier, self.solver
        from .pymoto_oracle import cg_solve, vcycle
        orig_update = LinSolveOracle.update

        def update(A):
            levels = solver.levels
            solver.levels = 0      # skip the uncached hierarchy build, keep the LDA bookkeeping
            try:
                solver.A = A
                d = A.diagonal()
                nz = A.copy()
                nz.eliminate_zeros()
                nnz_row = np.diff(nz.indptr)
                nnz_col = np.asarray((nz != 0).sum(axis=0)).ravel()
                diag_only = (d != 0) & (nnz_row <= 1) & (nnz_col <= 1)
                solver.idia = np.nonzero(diag_only)[0]
                solver.isel = np.nonzero(~diag_only)[0]
                solver.xs, solver.bs = [], []
                lv = hier.update(A)
                solver._inner = lambda b, x0: cg_solve(A, b, lambda r: vcycle(lv[0], r), x0, solver.tol, solver.maxit,
                                                       solver.restart)
            finally:
                solver.levels = levels
        solver.update = update
        del orig_update

    def step(self):
        """filter -> SIMP -> assemble -> MG setup -> CG -> compliance -> sensitivity -> OC; returns c."""
        g, x = self.grid, self.x
        xf = conv_filter(g, self.W, x)
        xs = simp(xf)
        K = self.csr.assemble(xs)
        u = self.solver.response(K, self.f)
        c = float(self.f @ u)
        lam = self.solver.adjoint(self.f)
        dxs = sensitivity_contract(g, self.K0, [-lam], [u], self.bc)
        dx = conv_filter_T(g, self.W, dxs * simp_derivative(xf))
        self.x = oc_step(x, dx, self.volfrac, move=self.move)
        return c


def cantilever_loads(grid):
    """The cantilever of the examples: face i = 0 clamped (all components), unit -y load at the middle node of
    the face i = nelx (examples/topology_optimization/ex_compliance_multigrid.py:81-100)."""
    g = grid
    nodes = g.nodes_where(i=0)
    bc = (nodes[:, None] * g.dim + np.arange(g.dim)).ravel()
    f = np.zeros(g.ndof)
    tip = g.node_number(g.nelx, g.nely // 2, g.nelz // 2)
    f[g.dim * tip + 1] = -1.0
    return bc, f


def fp64_cg_reference(shape, x, radius=2.5, levels=4, w=0.6, smooth_steps=2, tol=1e-12, maxit=5000):
    """pyMOTO's FP64 path for one design of the cantilever: FilterConv (filter.py:8-220), SIMP, assembly
    (assembly.py:245-296), CG (iterative.py:295-403) preconditioned by the geometric multigrid V-cycle
    (iterative.py:124-256, damped Jacobi, SuperLU on the coarsest level) until the recursive relative residual
    is below `tol`, the compliance f.u and its adjoint sensitivity dc/dx (assembly.py:298-315, the filter's
    transpose).  Returns a dict with c, u, dc, the true relative residual and the CG iteration count."""
    g = Grid(*shape)
    bc, f = cantilever_loads(g)
    K0 = element_stiffness(g)
    W = conv_filter_weights(g, radius)
    xf = conv_filter(g, W, x)
    xs = simp(xf)
    K = StructuredCSR(g, K0, bc).assemble(xs)
    hier = CachedHierarchy(g, levels, w, smooth_steps).update(K)
    u, it, _ = cg_solve(K, f, lambda r: vcycle(hier[0], r), None, tol, maxit, 50)
    res = relative_residual(K, u, f)
    dxs = sensitivity_contract(g, K0, [-u], [u], bc)
    dc = conv_filter_T(g, W, dxs * simp_derivative(xf))
    return {"c": float(f @ u), "u": u, "dc": dc, "residual": float(res), "iterations": int(it) + 1, "bc": bc, "f": f}
