"""numpy/scipy restatement of pyMOTO's structured-grid compliance path (test infrastructure only).

Every function names the pyMOTO v2.0.1 source it follows (paths relative to the pyMOTO project).
FP64 throughout, like the reference.  The oracle is the checker for the CUDA library and the timed
CPU baseline; it is never imported by the product package.
"""
import warnings

import numpy as np
import scipy.sparse as sps
from scipy.sparse.linalg import splu

__all__ = [
    "Grid", "element_stiffness", "material_matrix", "assemble", "default_bcdiagval",
    "density_filter_matrix", "density_filter_nonpadding", "density_filter", "density_filter_T",
    "conv_filter_weights", "conv_filter_index_map", "conv_filter", "conv_filter_T",
    "simp", "simp_derivative", "prolongation", "MGLevel", "build_hierarchy", "vcycle",
    "cg_solve", "LinSolveOracle", "sensitivity_contract", "oc_step", "direct_solve",
    "CompliancePipeline", "relative_residual",
]

# Local node order of a voxel element, as sign triples (pymoto/common/domain.py:132-142).
_LOCAL_SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [-1, 1, -1], [1, 1, -1],
                         [-1, -1, 1], [1, -1, 1], [-1, 1, 1], [1, 1, 1]], dtype=np.int64)


class Grid:
    """Structured voxel numbering (pymoto/common/domain.py:102-164, 200-251, 338-362).

    element (i,j,k) -> (k*nely + j)*nelx + i; node (i,j,k) -> (k*(nely+1) + j)*(nelx+1) + i;
    dof -> node*dim + d.  2D grids have nelz == 0 and use the first four local nodes.
    """

    def __init__(self, nelx, nely, nelz=0, unitx=1.0, unity=1.0, unitz=1.0):
        self.nelx, self.nely, self.nelz = int(nelx), int(nely), int(nelz)
        self.dim = 2 if self.nelz == 0 else 3
        self.unit = np.array([unitx, unity, unitz], dtype=np.float64)
        self.nel = self.nelx * self.nely * max(self.nelz, 1)
        self.nnodes = (self.nelx + 1) * (self.nely + 1) * (self.nelz + 1)
        self.elemnodes = 2 ** self.dim
        self.ndof = self.nnodes * self.dim

    @property
    def shape(self):
        return (self.nelx, self.nely) if self.dim == 2 else (self.nelx, self.nely, self.nelz)

    def elem_number(self, i, j, k=0):
        return (np.asarray(k) * self.nely + j) * self.nelx + i

    def node_number(self, i, j, k=0):
        return (np.asarray(k) * (self.nely + 1) + j) * (self.nelx + 1) + i

    def elem_ijk(self):
        e = np.arange(self.nel, dtype=np.int64)
        return e % self.nelx, (e // self.nelx) % self.nely, e // (self.nelx * self.nely)

    def conn(self):
        """Node connectivity (nel, 2**dim), local order of domain.py:132-142 / :338-351."""
        i, j, k = self.elem_ijk()
        offs = (_LOCAL_SIGNS[: self.elemnodes] > 0).astype(np.int64)
        return np.stack([self.node_number(i + o[0], j + o[1], k + o[2]) for o in offs], axis=-1)

    def dofconn(self, ndof=None):
        """Dof connectivity (nel, 2**dim * ndof), domain.py:353-362."""
        ndof = self.dim if ndof is None else ndof
        c = self.conn()
        return (c[:, :, None] * ndof + np.arange(ndof)[None, None, :]).reshape(c.shape[0], -1)

    def coarse(self):
        """Half-resolution grid with doubled element size (pymoto/solvers/iterative.py:153-155)."""
        if self.nelx % 2 or self.nely % 2 or self.nelz % 2:
            raise ValueError(f"grid {self.shape} is not divisible by 2")
        return Grid(self.nelx // 2, self.nely // 2, self.nelz // 2, *(2.0 * self.unit))

    def nodes_where(self, i=None, j=None, k=None):
        """Node numbers of the nodes whose index equals the given values (None = all)."""
        ii = np.arange(self.nelx + 1) if i is None else np.atleast_1d(i)
        jj = np.arange(self.nely + 1) if j is None else np.atleast_1d(j)
        kk = np.arange(self.nelz + 1) if k is None else np.atleast_1d(k)
        I, J, K = np.meshgrid(ii, jj, kk, indexing="ij")
        return self.node_number(I, J, K).ravel()


# --------------------------------------------------------------------------- element stiffness
def material_matrix(E, nu, mode):
    """Isotropic constitutive matrix (pymoto/modules/assembly.py:373-404)."""
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    c1 = 2.0 * mu + lam
    mode = mode.lower()
    if "strain" in mode:
        return np.array([[c1, lam, 0.0], [lam, c1, 0.0], [0.0, 0.0, mu]])
    if "stress" in mode:
        a = E / (1.0 - nu * nu)
        return a * np.array([[1.0, nu, 0.0], [nu, 1.0, 0.0], [0.0, 0.0, (1.0 - nu) / 2.0]])
    if "3d" in mode:
        D = np.zeros((6, 6))
        D[:3, :3] = lam
        D[np.arange(3), np.arange(3)] = c1
        D[np.arange(3, 6), np.arange(3, 6)] = mu
        return D
    raise ValueError(mode)


def _shape_derivatives(grid, pos):
    """dN/dx at a point inside an element (pymoto/common/domain.py:409-428)."""
    dim, nn = grid.dim, grid.elemnodes
    s = _LOCAL_SIGNS[:nn]
    dN = np.full((dim, nn), 1.0 / np.prod(grid.unit[:dim]))
    for a in range(dim):
        for b in range(dim):
            if a != b:
                dN[a] *= grid.unit[b] / 2.0 + s[:, b] * pos[b]
        dN[a] *= s[:, a]
    return dN


def _strain_matrix(dN):
    """Strain-displacement matrix, Voigt order (pymoto/modules/assembly.py:318-370)."""
    dim, nn = dN.shape
    if dim == 2:
        B = np.zeros((3, 2 * nn))
        B[0, 0::2] = dN[0]
        B[1, 1::2] = dN[1]
        B[2, 0::2] = dN[1]
        B[2, 1::2] = dN[0]
        return B
    B = np.zeros((6, 3 * nn))
    B[0, 0::3] = dN[0]
    B[1, 1::3] = dN[1]
    B[2, 2::3] = dN[2]
    B[3, 1::3] = dN[2]
    B[3, 2::3] = dN[1]
    B[4, 0::3] = dN[2]
    B[4, 2::3] = dN[0]
    B[5, 0::3] = dN[1]
    B[5, 1::3] = dN[0]
    return B


def element_stiffness(grid, e_modulus=1.0, poisson_ratio=0.3, plane="strain"):
    """Element stiffness by 2x2(x2) Gauss quadrature (pymoto/modules/assembly.py:427-463)."""
    D = material_matrix(e_modulus, poisson_ratio, "3d" if grid.dim == 3 else plane)
    w = np.prod(grid.unit[: grid.dim] / 2.0)
    if grid.dim == 2:
        w *= grid.unit[2]
    nd = grid.elemnodes * grid.dim
    K0 = np.zeros((nd, nd))
    for s in _LOCAL_SIGNS[: grid.elemnodes]:
        pos = s * (grid.unit / 2.0) / np.sqrt(3.0)
        B = _strain_matrix(_shape_derivatives(grid, pos))
        K0 += w * (B.T @ D @ B)
    return K0


def default_bcdiagval(K0):
    """Diagonal value placed on constrained rows: max entry of the element matrix (assembly.py:94-98)."""
    return float(np.max(K0))


# --------------------------------------------------------------------------- assembly
def assemble(grid, K0, x, bc=None, bcdiagval=None, ndof=None):
    """K = sum_e x_e K0 with Dirichlet rows/cols zeroed and bcdiagval on their diagonal.

    Same matrix as pymoto/modules/assembly.py:245-296 (BC data redirected at :210-230, diagonal set at
    :272); built here through COO summation instead of the precomputed datamap.  ndof: dofs per node (default
    the grid's dimension; 1 for AssemblePoisson and AssembleMass(ndof=1), assembly.py:466-560).
    """
    dc = grid.dofconn(ndof)
    nd = dc.shape[1]
    rows = np.repeat(dc, nd, axis=1).ravel()
    cols = np.tile(dc, (1, nd)).ravel()
    vals = (x.reshape(-1, 1) * K0.reshape(1, -1)).ravel()
    n = grid.nnodes * (grid.dim if ndof is None else ndof)
    if bc is not None and len(bc) > 0:
        bc = np.asarray(bc).ravel()
        isbc = np.zeros(n, dtype=bool)
        isbc[bc] = True
        keep = ~(isbc[rows] | isbc[cols])
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
        bcdiagval = default_bcdiagval(K0) if bcdiagval is None else bcdiagval
        rows = np.concatenate([rows, bc])
        cols = np.concatenate([cols, bc])
        vals = np.concatenate([vals, np.full(bc.size, bcdiagval)])
    K = sps.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    K.sum_duplicates()
    return K


def sensitivity_contract(grid, K0, u_list, v_list, bc=None, ndof=None):
    """dx_e = sum_k u_k[dofs_e]^T K0 v_k[dofs_e] with constrained rows/cols of the dyad zeroed.

    pymoto/modules/assembly.py:298-315 with DyadicMatrix.contract (pymoto/common/dyadcarrier.py:366-414)
    and the row/column zeroing of dyadcarrier.py:179-189.  ndof: dofs per node (default the grid's dimension).
    """
    dc = grid.dofconn(ndof)
    out = np.zeros(grid.nel)
    for u, v in zip(u_list, v_list):
        u = np.array(u, dtype=np.float64, copy=True)
        v = np.array(v, dtype=np.float64, copy=True)
        if bc is not None:
            u[bc] = 0.0
            v[bc] = 0.0
        out += np.einsum("ei,ij,ej->e", u[dc], K0, v[dc], optimize=True)
    return out


# --------------------------------------------------------------------------- filters
def density_filter_matrix(grid, radius):
    """H_ij = max(0, r - |c_i - c_j|) over a (2*int(r)+1)^dim window (pymoto/modules/filter.py:314-378).

    Returns (H as CSR, row sums s) so that y = H x / s (filter.py:247-270).  Distances are in element
    index units, as in the reference.
    """
    d = int(radius)
    nx, ny, nz = grid.nelx, grid.nely, max(grid.nelz, 1)
    I, J, K = grid.elem_ijk()
    rows, cols, vals = [], [], []
    dzr = range(-d, d + 1) if grid.dim == 3 else [0]
    for dz in dzr:
        for dy in range(-d, d + 1):
            for dx in range(-d, d + 1):
                i2, j2, k2 = I + dx, J + dy, K + dz
                ok = (i2 >= 0) & (i2 < nx) & (j2 >= 0) & (j2 < ny) & (k2 >= 0) & (k2 < nz)
                rows.append(np.nonzero(ok)[0])
                cols.append(grid.elem_number(i2[ok], j2[ok], k2[ok]))
                vals.append(np.full(ok.sum(), max(0.0, radius - np.sqrt(dx * dx + dy * dy + dz * dz))))
    H = sps.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(grid.nel, grid.nel)).tocsr()
    s = np.asarray(H.sum(axis=1)).ravel()
    return H, s


def density_filter_nonpadding(s, nonpadding):
    """Row sums with `nonpadding`: rows outside it take max(s), which mimics zero densities outside the
    domain (pymoto/modules/filter.py:241-255)."""
    s = s.copy()
    s[~np.isin(np.arange(s.size), nonpadding)] = s.max()
    return s


def density_filter(H, s, x):
    """y = H x / s (pymoto/modules/filter.py:266-267)."""
    return (H @ x) / s


def density_filter_T(H, s, dy):
    """Adjoint H^T (dy / s); H is symmetric (pymoto/modules/filter.py:269-270)."""
    return H.T @ (dy / s)


def conv_filter_weights(grid, radius):
    """Normalised cone kernel of FilterConv (pymoto/modules/filter.py:189-205, relative units)."""
    nx, ny, nz = grid.nelx, grid.nely, grid.nelz
    dx = min(nx, int(radius - 1e-10))
    dy = min(ny, int(radius - 1e-10))
    dz = min(nz, int(radius - 1e-10))
    X, Y, Z = np.meshgrid(np.arange(-dx, dx + 1.0), np.arange(-dy, dy + 1.0), np.arange(-dz, dz + 1.0),
                          indexing="ij")
    w = np.maximum(0.0, radius - np.sqrt(X * X + Y * Y + Z * Z))
    return w / np.sum(w)


def conv_filter_index_map(grid, weights):
    """Element numbers of the symmetric-padded grid, shape (nx+2px, ny+2py, nz+2pz).

    The padding follows numpy's 'symmetric' mode per axis (pymoto/modules/filter.py:98-160, default BCs).
    """
    pads = [s // 2 for s in weights.shape]
    sizes = [grid.nelx, grid.nely, max(grid.nelz, 1)]
    maps = [np.pad(np.arange(n), p, mode="symmetric") for n, p in zip(sizes, pads)]
    I, J, K = np.meshgrid(*maps, indexing="ij")
    return grid.elem_number(I, J, K)


def conv_filter(grid, weights, x):
    """Padded 'valid' convolution y = W * x_pad (pymoto/modules/filter.py:207-212)."""
    pad_map = conv_filter_index_map(grid, weights)
    xp = x[pad_map]
    sx, sy, sz = grid.nelx, grid.nely, max(grid.nelz, 1)
    kx, ky, kz = weights.shape
    y3 = np.zeros((sx, sy, sz))
    for a in range(kx):
        for b in range(ky):
            for c in range(kz):
                # convolution flips the kernel: output o reads x_pad[o + (k-1) - m]
                y3 += weights[kx - 1 - a, ky - 1 - b, kz - 1 - c] * xp[a:a + sx, b:b + sy, c:c + sz]
    I, J, K = np.meshgrid(np.arange(sx), np.arange(sy), np.arange(sz), indexing="ij")
    y = np.zeros(grid.nel)
    y[grid.elem_number(I, J, K).ravel()] = y3.ravel()
    return y


def conv_filter_T(grid, weights, dy):
    """Adjoint of conv_filter: full correlation then accumulation through the pad map (filter.py:214-220)."""
    pad_map = conv_filter_index_map(grid, weights)
    sx, sy, sz = grid.nelx, grid.nely, max(grid.nelz, 1)
    kx, ky, kz = weights.shape
    I, J, K = np.meshgrid(np.arange(sx), np.arange(sy), np.arange(sz), indexing="ij")
    d3 = dy[grid.elem_number(I, J, K)]
    gp = np.zeros(pad_map.shape)
    for a in range(kx):
        for b in range(ky):
            for c in range(kz):
                gp[a:a + sx, b:b + sy, c:c + sz] += weights[kx - 1 - a, ky - 1 - b, kz - 1 - c] * d3
    dx = np.zeros(grid.nel)
    np.add.at(dx, pad_map.ravel(), gp.ravel())
    return dx


# --------------------------------------------------------------------------- SIMP
def simp(x, xmin=1e-9, penal=3.0):
    """xmin + (1 - xmin) x^p, the MathExpression used by the compliance examples
    (pymoto/modules/generic.py:94-99; examples/topology_optimization/ex_compliance.py:89)."""
    return xmin + (1.0 - xmin) * x ** penal


def simp_derivative(x, xmin=1e-9, penal=3.0):
    """d/dx of simp (pymoto/modules/generic.py:101-140 via the symbolic derivative)."""
    return penal * (1.0 - xmin) * x ** (penal - 1.0)


# --------------------------------------------------------------------------- multigrid
def prolongation(grid, ndof=None):
    """Trilinear prolongation R (fine dofs x coarse dofs), pymoto/solvers/iterative.py:178-220.

    Fine node (2I+a, 2J+b, 2K+c) receives weight prod(1 if offset 0 else 1/2) from coarse node (I,J,K), for each
    of the ndof dofs of the node (default the grid's dimension).
    """
    cg = grid.coarse()
    nd = grid.dim if ndof is None else ndof
    rows, cols, vals = [], [], []
    offs_k = [-1, 0, 1] if grid.dim == 3 else [0]
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            for c in offs_k:
                ci = np.arange(max(-a, 0), min(cg.nelx + 1 - a, cg.nelx + 1))
                cj = np.arange(max(-b, 0), min(cg.nely + 1 - b, cg.nely + 1))
                ck = np.arange(max(-c, 0), min(cg.nelz + 1 - c, cg.nelz + 1))
                CI, CJ, CK = np.meshgrid(ci, cj, ck, indexing="ij")
                nc = cg.node_number(CI, CJ, CK).ravel()
                nf = grid.node_number(2 * CI + a, 2 * CJ + b, 2 * CK + c).ravel()
                w = (0.5 if a else 1.0) * (0.5 if b else 1.0) * (0.5 if c else 1.0)
                for d in range(nd):
                    rows.append(nf * nd + d)
                    cols.append(nc * nd + d)
                    vals.append(np.full(nf.size, w))
    R = sps.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(grid.nnodes * nd, cg.nnodes * nd)).tocsr()
    return R


class MGLevel:
    """One geometric-multigrid level (pymoto/solvers/iterative.py:124-256) with a damped-Jacobi smoother
    (iterative.py:21-47).  ``inner`` is the next MGLevel or None for the direct coarsest solve."""

    def __init__(self, grid, A, w=0.5, smooth_steps=5, ndof=None):
        self.grid, self.A, self.w, self.smooth_steps = grid, A, w, smooth_steps
        self.D = A.diagonal()
        self.R = prolongation(grid, ndof)
        self.Ac = (self.R.T @ A @ self.R).tocsr()
        self.inner = None
        self.lu = None


def build_hierarchy(grid, A, levels, w=0.5, smooth_steps=5, ndof=None):
    """Chain of GeometricMultigrid levels; the last Galerkin operator gets a direct LU factorisation
    (SuperLU, pymoto/solvers/sparse.py:515-555, chosen by auto_determine.py:109-122).  ndof: dofs per node
    (default the grid's dimension)."""
    lvls = []
    g, M = grid, A
    for _ in range(levels - 1):
        lv = MGLevel(g, M, w, smooth_steps, ndof)
        if lvls:
            lvls[-1].inner = lv
        lvls.append(lv)
        g, M = g.coarse(), lv.Ac
    lvls[-1].lu = splu(lvls[-1].Ac.tocsc())
    return lvls


def vcycle(lv, rhs, x0=None):
    """V-cycle of pymoto/solvers/iterative.py:222-256 (smoother = w * r / D)."""
    A, D, w = lv.A, lv.D, lv.w
    if x0 is None:
        u = w * (rhs / D)
    else:
        u = x0 + w * ((rhs - A @ x0) / D)
    for _ in range(lv.smooth_steps - 1):
        u = u + w * ((rhs - A @ u) / D)
    r = rhs - A @ u
    rc = lv.R.T @ r
    uc = vcycle(lv.inner, rc) if lv.inner is not None else lv.lu.solve(rc)
    u = u + lv.R @ uc
    for _ in range(lv.smooth_steps):
        u = u + w * ((rhs - A @ u) / D)
    return u


def relative_residual(A, x, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(A @ x - b) / (nb if nb != 0 else 1.0)


def cg_solve(A, b, precond=None, x0=None, tol=1e-7, maxit=10000, restart=50):
    """Single right-hand-side form of the block PCG of pymoto/solvers/iterative.py:340-403.

    Returns (x, iterations, final recursive relative residual).  ``precond`` maps r -> z.
    """
    M = (lambda r: r.copy()) if precond is None else precond
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    bn = np.linalg.norm(b)
    r = b - A @ x
    tval = np.linalg.norm(r) / bn
    if tval <= tol:
        return x, 0, tval
    z = M(r)
    p = z / np.sqrt(z @ z)                       # orth(z, normalize=True), iterative.py:259-292
    it = 0
    for it in range(maxit):
        q = A @ p
        pq = p @ q
        alpha = (p @ r) / pq
        x = x + alpha * p
        if it % restart == 0:                    # explicit residual, iterative.py:381-384
            r = b - A @ x
        else:
            r = r - alpha * q
        tval = np.linalg.norm(r) / bn
        if tval <= tol:
            break
        z = M(r)
        beta = -(q @ z) / pq
        p = z + beta * p
    if tval > tol:
        warnings.warn(f"CG maximum iterations ({maxit}) reached, residual {tval}")
    return x, it, tval


def direct_solve(A, b):
    """FP64 sparse LU solve (SuperLU), the reference's direct solver (pymoto/solvers/sparse.py:533-555)."""
    return splu(A.tocsc()).solve(b)


class LinSolveOracle:
    """LinSolve + LDAWrapper semantics (pymoto/modules/linalg.py:164-219, pymoto/solvers/solvers.py:140-306)
    for a symmetric stiffness matrix with an MG-preconditioned CG (or a direct solve when levels == 0).

    * diagonal-only rows (Dirichlet dofs) are solved directly as rhs/diag (solvers.py:174-176);
    * the solve is warm-started from the previous solution with those rows zeroed (linalg.py:195,
      solvers.py:210-217);
    * each new solution is stored as a normalised (x, A x) pair and later right-hand sides are first
      projected on the stored pairs (solvers.py:180-203, :233-248), which makes the compliance adjoint free;
    * the wrapper tolerance is 5 x the CG tolerance (linalg.py:185-189).
    """

    def __init__(self, grid=None, levels=0, w=0.5, smooth_steps=5, tol=1e-7, maxit=10000, restart=50):
        self.grid, self.levels, self.w, self.smooth_steps = grid, levels, w, smooth_steps
        self.tol, self.maxit, self.restart = tol, maxit, restart
        self.lda_tol = 5.0 * tol if levels > 0 else 1e-7
        self.u = None
        self.cg_iterations = []

    def update(self, A):
        self.A = A
        d = A.diagonal()
        nnz_row = np.diff(A.indptr)
        nz = A.copy()
        nz.eliminate_zeros()
        nnz_row = np.diff(nz.indptr)
        nnz_col = np.asarray((nz != 0).sum(axis=0)).ravel()
        diag_only = (d != 0) & (nnz_row <= 1) & (nnz_col <= 1)     # solvers.py:88-96
        self.idia = np.nonzero(diag_only)[0]
        self.isel = np.nonzero(~diag_only)[0]
        self.xs, self.bs = [], []
        if self.levels > 0:
            self.hier = build_hierarchy(self.grid, A, self.levels, self.w, self.smooth_steps)
            self._inner = lambda b, x0: cg_solve(A, b, lambda r: vcycle(self.hier[0], r), x0, self.tol,
                                                 self.maxit, self.restart)
        else:
            lu = splu(A.tocsc())
            self._inner = lambda b, x0: (lu.solve(b), 0, 0.0)

    def solve(self, rhs, x0=None):
        A, isel, idia = self.A, self.isel, self.idia
        rl = np.array(rhs, dtype=np.float64, copy=True)
        sol = np.zeros_like(rl)
        sol[idia] = rl[idia] / A.diagonal()[idia]
        rl[idia] = 0.0
        for x, b in zip(self.xs, self.bs):
            alpha = (rl[isel] @ b) / (b @ b)
            rl[isel] -= alpha * b
            sol[isel] += alpha * x
        self.last_rtol = relative_residual(A, sol, rhs)
        if self.last_rtol > self.lda_tol:
            x0l = None
            if x0 is not None:
                x0l = np.array(x0, dtype=np.float64, copy=True)
                x0l[idia] = 0.0
                for x in self.xs:
                    x0l[isel] -= ((x0l[isel] @ x) / (x @ x)) * x
            xnew, its, _ = self._inner(rl, x0l)
            self.cg_iterations.append(its)
            sol[isel] += xnew[isel]
            xa = xnew[isel].copy()
            ba = (A @ xnew)[isel]
            for x, b in zip(self.xs, self.bs):
                beta = (ba @ b) / (b @ b)
                ba = ba - beta * b
                xa = xa - beta * x
            bn = np.linalg.norm(ba)
            if np.isfinite(bn) and bn != 0:
                self.xs.append(xa / bn)
                self.bs.append(ba / bn)
        return sol

    def response(self, A, f):
        self.update(A)
        self.u = self.solve(f, x0=self.u)
        return self.u

    def adjoint(self, dfdu):
        return self.solve(dfdu)


# --------------------------------------------------------------------------- optimizer
def oc_step(x, dg, maxvol, move=0.1, xmin=0.0, xmax=1.0, l1=0.0, l2=1e5, l1l2tol=1e-4):
    """Optimality-criteria bisection (pymoto/common/optimizers.py:402-437).  ``maxvol`` is the volume
    fraction; the returned design is the one of the last bisection step, as in the reference."""
    dg = np.minimum(dg, 0.0)
    lb = np.maximum(xmin, x - move)
    ub = np.minimum(xmax, x + move)
    xnew = x.copy()
    while l2 - l1 > l1l2tol:
        lmid = 0.5 * (l1 + l2)
        xnew = np.clip(x * np.sqrt(-dg / lmid), lb, ub)
        if np.sum(xnew) - maxvol * x.size > 0:
            l1 = lmid
        else:
            l2 = lmid
    return xnew


# --------------------------------------------------------------------------- whole pipeline
class CompliancePipeline:
    """filter -> SIMP -> assemble -> LinSolve -> c = f.u and the reverse sweep, as the network of
    examples/topology_optimization/ex_compliance.py:76-137 / ex_compliance_multigrid.py:81-162 builds it."""

    def __init__(self, grid, bc, f, filter_kind="density", radius=1.5, xmin=1e-9, penal=3.0,
                 e_modulus=1.0, poisson_ratio=0.3, plane="strain", levels=0, w=0.5, smooth_steps=5,
                 tol=1e-7, maxit=10000):
        self.grid, self.bc, self.f = grid, np.asarray(bc), np.asarray(f, dtype=np.float64)
        self.xmin, self.penal = xmin, penal
        self.K0 = element_stiffness(grid, e_modulus, poisson_ratio, plane)
        self.filter_kind = filter_kind
        if filter_kind == "density":
            self.H, self.Hs = density_filter_matrix(grid, radius)
        else:
            self.W = conv_filter_weights(grid, radius)
        self.solver = LinSolveOracle(grid, levels, w, smooth_steps, tol, maxit)

    def filt(self, x):
        if self.filter_kind == "density":
            return density_filter(self.H, self.Hs, x)
        return conv_filter(self.grid, self.W, x)

    def filt_T(self, d):
        if self.filter_kind == "density":
            return density_filter_T(self.H, self.Hs, d)
        return conv_filter_T(self.grid, self.W, d)

    def response(self, x):
        self.xf = self.filt(x)
        self.xs = simp(self.xf, self.xmin, self.penal)
        self.K = assemble(self.grid, self.K0, self.xs, self.bc)
        self.u = self.solver.response(self.K, self.f)
        self.c = float(self.f @ self.u)
        return self.c

    def sensitivity(self):
        lam = self.solver.adjoint(self.f)                   # dc/du = f (generic.py:214-225)
        dxs = sensitivity_contract(self.grid, self.K0, [-lam], [self.u], self.bc)
        dxf = dxs * simp_derivative(self.xf, self.xmin, self.penal)
        return self.filt_T(dxf)
