"""Kernel-by-kernel parity of libpymoto_gb300 against the oracle and the golden vectors (GPU)."""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

import oracle as O
from conftest import clamp_face_dofs

pytestmark = pytest.mark.gpu

SHAPES = [(6, 4, 0), (4, 3, 2), (8, 6, 4), (7, 5, 3)]


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def host(t):
    return t.double().cpu().numpy()


@pytest.fixture(scope="module")
def pg():
    import pymoto_gb300 as pg
    from pymoto_gb300 import _lib
    _lib.load()
    return pg


def _setup(pg, shape, seed=0, bc=True):
    from pymoto_gb300.operators import bc_node_mask
    g = O.Grid(*shape)
    rng = np.random.default_rng(seed)
    x = rng.uniform(1e-3, 1.0, g.nel) ** 3
    bcd = clamp_face_dofs(g) if bc else np.zeros(0, dtype=np.int64)
    K0 = O.element_stiffness(g)
    K = O.assemble(g, K0, x, bcd)
    mask = dev(bc_node_mask(g.nnodes, g.dim, bcd), torch.uint8)
    op = pg.StiffnessOperator(pg.Grid(*shape), dev(x), K0, mask, O.default_bcdiagval(K0))
    return g, K, op, rng


@pytest.mark.parametrize("shape", SHAPES)
def test_dof_connectivity_bit_exact(pg, shape):
    from pymoto_gb300._lib import call, stream
    g = O.Grid(*shape)
    dc = torch.empty((g.nel, g.elemnodes * g.dim), dtype=torch.int64, device="cuda")
    call("pmg_dof_connectivity", *shape, dc, stream())
    assert np.array_equal(dc.cpu().numpy(), g.dofconn())


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("bc", [True, False])
def test_matvec_fp64_matches_csr(pg, shape, bc):
    g, K, op, rng = _setup(pg, shape, bc=bc)
    u = rng.standard_normal(g.ndof)
    y = host(op.matvec(dev(u)))
    ref = K @ u
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    np.testing.assert_allclose(host(op.diagonal()), K.diagonal(), rtol=1e-14)


@pytest.mark.parametrize("shape", SHAPES)
def test_fp64_stencil_and_matrix_free_agree(pg, shape):
    """The two FP64 product paths (assembled level-0 stencil, matrix-free gather) give the same K u."""
    from pymoto_gb300._lib import JACOBI
    g, K, op, rng = _setup(pg, shape, seed=5)
    u, b = rng.standard_normal(g.ndof), rng.standard_normal(g.ndof)
    ys = host(op.matvec(dev(u)))
    js = host(op.apply(JACOBI, dev(u), dev(b), op.diagonal(), 0.6))
    op.fp64_stencil = False
    ym = host(op.matvec(dev(u)))
    jm = host(op.apply(JACOBI, dev(u), dev(b), op.diagonal(), 0.6))
    np.testing.assert_allclose(ys, ym, rtol=0, atol=1e-13 * np.abs(ym).max())
    np.testing.assert_allclose(js, jm, rtol=1e-12, atol=1e-12 * np.abs(jm).max())


@pytest.mark.parametrize("code", ["f64", "f32"])
def test_stencil_row_and_split_kernels(pg, code):
    """Stencil products on both sides of the split-row threshold (2^16 rows): the fine level (263,835 rows,
    one thread per row) against the matrix-free product, and its Galerkin level (35,343 rows, split rows)
    against R^T (K (R u)) through the fine level, in all four modes."""
    from pymoto_gb300._lib import F32, F64, JACOBI, RESIDUAL, call, stream
    shape = (64, 32, 40)
    rng = np.random.default_rng(3)
    g = pg.Grid(*shape)
    x = dev(rng.uniform(1e-3, 1.0, g.nel) ** 3)
    gg = O.Grid(*shape)
    K0 = O.element_stiffness(gg)
    mask = torch.zeros(g.nnodes, dtype=torch.uint8, device="cuda")
    op = pg.StiffnessOperator(g, x, K0, mask, O.default_bcdiagval(K0))
    c = F64 if code == "f64" else F32
    dt = torch.float64 if code == "f64" else torch.float32
    tol = 1e-12 if code == "f64" else 2e-5
    if code == "f32":
        op = op.astype(F32)
    # fine level: assembled stencil (row kernel) vs the matrix-free product of the same operator
    S = op.stencil() if code == "f64" else None
    u = torch.randn(g.ndof, dtype=dt, device="cuda")
    b = torch.randn_like(u)
    if code == "f64":
        y_row = torch.empty_like(u)
        call("pmg_stencil_apply", 0, c, *shape, S, u, b, u, 0.0, y_row, stream())
        y_mf = op.matvec(u)
        assert float((y_row - y_mf).abs().max()) <= tol * float(y_mf.abs().max())
    # coarse level (split kernel) vs restriction of the fine product of the prolonged vector
    A1 = op.galerkin()
    gc = A1.grid
    uc = torch.randn(gc.ndof, dtype=dt, device="cuda")
    bc = torch.randn_like(uc)
    uf = torch.zeros(g.ndof, dtype=dt, device="cuda")
    call("pmg_prolong_add", c, *shape, uc, uf, stream())
    kf = op.matvec(uf)
    ref = torch.empty_like(uc)
    call("pmg_restrict", c, *shape, kf, ref, stream())
    y = A1.matvec(uc)
    scale = float(ref.abs().max())
    assert float((y - ref).abs().max()) <= tol * scale
    D = A1.diagonal()
    r = A1.apply(RESIDUAL, uc, bc)
    assert float((r - (bc - ref)).abs().max()) <= tol * scale
    j = A1.apply(JACOBI, uc, bc, D, 0.6)
    jref = uc + 0.6 * ((bc - ref) / D)
    assert float((j - jref).abs().max()) <= tol * float(jref.abs().max()) * 10
    coef = torch.tensor([0.5, 0.7, 0.3, 0.9], dtype=torch.float64, device="cuda")
    d0 = torch.randn_like(uc)
    dd = d0.clone()
    yc = torch.empty_like(uc)
    assert A1.cheb_step(uc, bc, D, dd, coef, 1, out=yc) is not None
    dref = 0.3 * d0 + 0.9 * ((bc - ref) / D)
    assert float((dd - dref).abs().max()) <= tol * float(dref.abs().max()) * 10
    assert float((yc - (uc + dref)).abs().max()) <= tol * float((uc + dref).abs().max()) * 10


@pytest.mark.parametrize("shape", SHAPES)
def test_matvec_fp32_and_modes(pg, shape):
    from pymoto_gb300._lib import F32, JACOBI, RESIDUAL
    g, K, op, rng = _setup(pg, shape, seed=1)
    u, b = rng.standard_normal(g.ndof), rng.standard_normal(g.ndof)
    D = K.diagonal()
    r = host(op.apply(RESIDUAL, dev(u), dev(b)))
    np.testing.assert_allclose(r, b - K @ u, atol=1e-12 * np.abs(b - K @ u).max())
    jac = host(op.apply(JACOBI, dev(u), dev(b), op.diagonal(), 0.6))
    np.testing.assert_allclose(jac, u + 0.6 * ((b - K @ u) / D), rtol=1e-12, atol=1e-12)
    op32 = op.astype(F32)
    y32 = host(op32.matvec(dev(u, torch.float32)))
    ref = K @ u.astype(np.float32).astype(np.float64)
    assert np.abs(y32 - ref).max() <= 2e-6 * np.abs(ref).max()


@pytest.fixture(params=["fma", "tcgen05"])
def operator_kernel(request, pg):
    """Runs a test with each implementation of the FP32 3D operator selected, then restores the default."""
    prev = pg.set_operator_kernel(request.param)
    yield request.param
    pg.set_operator_kernel(prev)


# tiles of both kernels: several in x, y and z, ragged edges (the CUDA-core kernel's tile widths follow the node
# counts: 129 -> 5 x 26, 101 -> 4 x 26, 17 x 71 -> 17 x 15; the tensor-core kernel's tiles are 31 x 8 elements)
FP32_3D_SHAPES = [(40, 12, 10), (33, 9, 17), (64, 16, 8), (2, 2, 2),
                  (128, 8, 4), (100, 40, 6), (16, 70, 3), (1, 1, 1)]


@pytest.mark.parametrize("shape", FP32_3D_SHAPES)
@pytest.mark.parametrize("field", ["random", "smooth"])
def test_matvec_fp32_3d_tiles(pg, operator_kernel, shape, field):
    """FP32 3D operator, every implementation: all modes and the fused Chebyshev step against FP64 numpy.
    The smooth field sits on a large constant offset: K annihilates the offset, and the result must keep
    its accuracy relative to |K u|, not to |K| |u|.  Two applications give bitwise equal results."""
    from pymoto_gb300._lib import F32, JACOBI, RESIDUAL
    g, K, op, rng = _setup(pg, shape, seed=3)
    if field == "random":
        u = rng.standard_normal(g.ndof)
    else:
        nx, ny, nz = shape
        kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        base = np.stack([np.sin(0.3 * ii + 0.2 * jj), np.cos(0.25 * jj - 0.1 * kk), np.sin(0.2 * kk + 0.15 * ii)], -1)
        u = (1000.0 + base).reshape(-1)
    u = u.astype(np.float32).astype(np.float64)
    b = rng.standard_normal(g.ndof).astype(np.float32).astype(np.float64)
    op32 = op.astype(F32)
    D = op32.diagonal()
    ref = K @ u
    tol = (1e-5 if field == "random" else 1e-4) * np.abs(ref).max()
    y = op32.matvec(dev(u, torch.float32))
    assert np.abs(host(y) - ref).max() <= tol
    assert torch.equal(y, op32.matvec(dev(u, torch.float32)))
    r = host(op32.apply(RESIDUAL, dev(u, torch.float32), dev(b, torch.float32)))
    assert np.abs(r - (b - ref)).max() <= tol + 1e-6 * np.abs(b).max()
    Dh = host(D)
    jac = host(op32.apply(JACOBI, dev(u, torch.float32), dev(b, torch.float32), D, 0.6))
    jref = u + 0.6 * (b - ref) / Dh
    assert np.abs(jac - jref).max() <= 0.6 * (tol + 1e-6 * np.abs(b).max()) / np.abs(Dh).min() + 1e-6 * np.abs(u).max()
    # fused Chebyshev step 1: d <- a d + c (b - K u) / D, y = u + d
    d0 = rng.standard_normal(g.ndof).astype(np.float32).astype(np.float64)
    coef = torch.tensor([0.0, 0.5, 0.3, 0.9], dtype=torch.float64, device="cuda")
    dd = dev(d0, torch.float32)
    out = torch.empty_like(dd)
    op32.cheb_step(dev(u, torch.float32), dev(b, torch.float32), D, dd, coef, 1, out)
    dref = 0.3 * d0 + 0.9 * (b - ref) / Dh
    dtol = 0.9 * (tol + 1e-6 * np.abs(b).max()) / np.abs(Dh).min() + 1e-6 * np.abs(d0).max()
    assert np.abs(host(dd) - dref).max() <= dtol
    assert np.abs(host(out) - (u + dref)).max() <= dtol + 1e-6 * np.abs(u).max()


@pytest.mark.parametrize("unit,nu", [((1.0, 0.5, 2.0), 0.35), ((0.5, 0.5, 0.5), 0.2), ((1.0, 1.0, 1.0), 0.45)],
                         ids=["box", "cube-h0.5", "cube-nu0.45"])
def test_matvec_fp32_3d_element_shapes(pg, operator_kernel, unit, nu):
    """FP32 3D operator for box-shaped elements (the general K0 path of the CUDA-core kernel) and for cube
    elements of another size and Poisson ratio (its 10-value path), against the FP64 CSR matrix."""
    from pymoto_gb300._lib import F32
    from pymoto_gb300.operators import bc_node_mask
    shape = (20, 9, 7)
    g = O.Grid(*shape, unitx=unit[0], unity=unit[1], unitz=unit[2])
    rng = np.random.default_rng(8)
    x = rng.uniform(1e-3, 1.0, g.nel) ** 3
    bcd = clamp_face_dofs(g)
    K0 = O.element_stiffness(g, poisson_ratio=nu)
    K = O.assemble(g, K0, x, bcd)
    mask = dev(bc_node_mask(g.nnodes, g.dim, bcd), torch.uint8)
    op = pg.StiffnessOperator(pg.Grid(*shape), dev(x), K0, mask, O.default_bcdiagval(K0)).astype(F32)
    u = rng.standard_normal(g.ndof).astype(np.float32).astype(np.float64)
    ref = K @ u
    y = host(op.matvec(dev(u, torch.float32)))
    assert np.abs(y - ref).max() <= 1e-5 * np.abs(ref).max()


def test_matvec_golden(pg, golden):
    g = golden("assembly.npz")
    from pymoto_gb300.operators import bc_node_mask
    for tag in ["q4", "h8"]:
        shape = tuple(int(v) for v in g[f"{tag}_shape"]) + ((0,) if len(g[f"{tag}_shape"]) == 2 else ())
        grid = O.Grid(*shape)
        K0 = pg.element_stiffness(grid.dim)
        mask = dev(bc_node_mask(grid.nnodes, grid.dim, g[f"{tag}_bc"]), torch.uint8)
        op = pg.StiffnessOperator(pg.Grid(*shape), dev(g[f"{tag}_x"]), K0, mask, float(np.max(K0)))
        y = host(op.matvec(dev(g[f"{tag}_u"])))
        np.testing.assert_allclose(y, g[f"{tag}_Ku"], rtol=0, atol=1e-13 * np.abs(g[f"{tag}_Ku"]).max())


@pytest.mark.parametrize("shape", [(8, 4, 0), (6, 4, 2), (8, 6, 4)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_transfers_match_R(pg, shape, dtype):
    from pymoto_gb300._lib import call, dtype_code, stream
    g = O.Grid(*shape)
    R = O.prolongation(g)
    rng = np.random.default_rng(2)
    rf = rng.standard_normal(g.ndof)
    uc = rng.standard_normal(R.shape[1])
    uf0 = rng.standard_normal(g.ndof)
    rc = torch.empty(R.shape[1], dtype=dtype, device="cuda")
    call("pmg_restrict", dtype_code(rc), *shape, dev(rf, dtype), rc, stream())
    tol = 1e-14 if dtype == torch.float64 else 1e-6
    np.testing.assert_allclose(host(rc), R.T @ rf, rtol=0, atol=tol * np.abs(R.T @ rf).max())
    uf = dev(uf0, dtype)
    call("pmg_prolong_add", dtype_code(uf), *shape, dev(uc, dtype), uf, stream())
    np.testing.assert_allclose(host(uf), uf0 + R @ uc, rtol=0, atol=tol * np.abs(uf0 + R @ uc).max())


def _stencil_csr(op):
    """Assemble a StencilOperator into CSR via its dense matrix (test helper)."""
    return sps.csr_matrix(host(op.to_dense()))


@pytest.mark.parametrize("shape", [(8, 4, 0), (4, 4, 4), (8, 4, 4), (6, 4, 2)])
def test_galerkin_matches_RtKR(pg, shape):
    g, K, op, rng = _setup(pg, shape, seed=3)
    R = O.prolongation(g)
    Ac = (R.T @ K @ R).tocsr()
    A1 = op.galerkin()
    D1 = _stencil_csr(A1)
    scale = abs(Ac).max()
    assert abs(D1 - Ac).max() <= 1e-13 * scale
    # stencil apply and diagonal against the CSR product
    u = rng.standard_normal(Ac.shape[0])
    np.testing.assert_allclose(host(A1.matvec(dev(u))), Ac @ u, rtol=0, atol=1e-12 * np.abs(Ac @ u).max())
    np.testing.assert_allclose(host(A1.diagonal()), Ac.diagonal(), rtol=1e-13)
    # second level from element matrices
    gc = g.coarse()
    if gc.nelx % 2 == 0 and gc.nely % 2 == 0 and gc.nelz % 2 == 0 and gc.nelx >= 2 and gc.nely >= 2:
        R2 = O.prolongation(gc)
        Ac2 = (R2.T @ Ac @ R2).tocsr()
        D2 = _stencil_csr(A1.galerkin())
        assert abs(D2 - Ac2).max() <= 1e-12 * abs(Ac2).max()


def test_galerkin_golden(pg, golden):
    g = golden("multigrid.npz")
    from pymoto_gb300.operators import bc_node_mask
    for tag in ["q4", "h8", "h8b"]:
        s = [int(v) for v in g[f"{tag}_shape"]]
        shape = tuple(s + [0] * (3 - len(s)))
        grid = O.Grid(*shape)
        K0 = pg.element_stiffness(grid.dim)
        mask = dev(bc_node_mask(grid.nnodes, grid.dim, g[f"{tag}_bc"]), torch.uint8)
        op = pg.StiffnessOperator(pg.Grid(*shape), dev(g[f"{tag}_x"]), K0, mask, float(np.max(K0)))
        Ac = sps.csr_matrix((g[f"{tag}_Ac_data"], g[f"{tag}_Ac_indices"], g[f"{tag}_Ac_indptr"]))
        D1 = _stencil_csr(op.galerkin())
        Ac = sps.csr_matrix(Ac, shape=D1.shape)
        assert abs(D1 - Ac).max() <= 1e-13 * abs(Ac).max()


@pytest.mark.parametrize("n_shape", [(4, 2, 2), (8, 4, 4), (16, 8, 0), (50, 26, 0)])
def test_cholesky_banded(pg, n_shape):
    from pymoto_gb300._lib import call, stream
    g, K, op, rng = _setup(pg, n_shape, seed=4)
    A1 = op  # use a coarse Galerkin operator as the SPD test matrix where possible
    if O.Grid(*n_shape).nelx % 2 == 0 and n_shape[1] % 2 == 0 and n_shape[2] % 2 == 0:
        A1 = op.galerkin()
    Ad = A1.to_dense() if hasattr(A1, "to_dense") else None
    if Ad is None:
        pytest.skip("no stencil form")
    n = Ad.shape[0]
    bw = A1.bandwidth()
    An = host(Ad)
    Lf = Ad.clone()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("pmg_cholesky_factor", n, Lf, bw, info, stream())
    assert int(info.item()) == 0
    Lh = np.tril(host(Lf))
    # backward-stable factorisation: L L^T reproduces A to rounding
    assert np.abs(Lh @ Lh.T - An).max() <= 1e-13 * np.abs(An).max()
    b = rng.standard_normal(n)
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    call("pmg_cholesky_solve", 0, n, Lf, bw, dev(b), x, stream())
    xh = host(x)
    assert np.linalg.norm(An @ xh - b) <= 1e-12 * np.linalg.norm(An, 2) * np.linalg.norm(xh)
    ref = np.linalg.solve(An, b)
    assert np.linalg.norm(xh - ref) <= 1e-4 * np.linalg.norm(ref)
    # blocked substitution with the diagonal-tile inverses, FP64 and FP32
    nblk = (n + 31) // 32
    Lh_full = np.tril(Lh)
    for code, dt in [(0, torch.float64), (1, torch.float32)]:
        Dinv = torch.empty(nblk * 32 * 32, dtype=dt, device="cuda")
        call("pmg_cholesky_block_inverses", code, n, Lf, Dinv, stream())
        D = host(Dinv).reshape(nblk, 32, 32)
        for kb in range(nblk):
            k0, nb = 32 * kb, min(32, n - 32 * kb)
            blk = Lh_full[k0:k0 + nb, k0:k0 + nb]
            tol = 1e-12 if code == 0 else 1e-6
            assert np.abs(D[kb, :nb, :nb] @ blk - np.eye(nb)).max() <= tol * max(1.0, np.abs(D[kb]).max() * np.abs(blk).max())
            assert np.abs(D[kb, nb:, :]).max(initial=0.0) == 0.0 and np.abs(D[kb, :, nb:]).max(initial=0.0) == 0.0
        Ld = Lf.to(dt)
        xb = torch.empty(n, dtype=dt, device="cuda")
        call("pmg_cholesky_solve_blocked", code, n, Ld, bw, Dinv, dev(b, dt), xb, stream())
        xbh = host(xb)
        if code == 0:
            assert np.linalg.norm(An @ xbh - b) <= 1e-12 * np.linalg.norm(An, 2) * np.linalg.norm(xbh)
        else:
            # FP32 substitution with the rounded factor: backward error at FP32 level
            Lr = np.tril(host(Ld))
            assert np.linalg.norm(Lr @ (Lr.T @ xbh) - host(dev(b, dt))) <= 1e-4 * np.linalg.norm(Lr, 2) ** 2 * np.linalg.norm(xbh)


@pytest.mark.parametrize("n_shape", [(8, 4, 4), (16, 8, 0)])
def test_cholesky_inverse_and_gemv(pg, n_shape):
    from pymoto_gb300._lib import call, stream
    g, K, op, rng = _setup(pg, n_shape, seed=9)
    A1 = op.galerkin()
    Ad = A1.to_dense()
    n, bw = Ad.shape[0], A1.bandwidth()
    An = host(Ad)
    L = Ad.clone()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("pmg_cholesky_factor", n, L, bw, info, stream())
    Ainv = torch.empty_like(L)
    call("pmg_cholesky_inverse", n, L, bw, Ainv, stream())
    Ai = host(Ainv)
    assert np.abs(Ai - Ai.T).max() <= 1e-10 * np.abs(Ai).max()
    assert np.abs(An @ Ai - np.eye(n)).max() <= 1e-8
    # FP32 inverse from the FP64 factor (tiles of L^{-1} in FP32, then L^{-T} L^{-1})
    from pymoto_gb300 import _lib
    scratch = torch.empty(_lib.load().pmg_cholesky_inverse_f32_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    Ai32 = torch.empty((n, n), dtype=torch.float32, device="cuda")
    call("pmg_cholesky_inverse_f32", n, L, bw, scratch, Ai32, stream())
    A32 = host(Ai32)
    rel = np.linalg.norm(A32 - Ai, 2) / np.linalg.norm(Ai, 2)
    kappa = np.linalg.cond(An)
    print(f"FP32 inverse: relative error {rel:.2e}, condition number {kappa:.2e}")
    assert rel <= max(1e-5, 1e-6 * np.sqrt(kappa))
    b = rng.standard_normal(n)
    for dt, tol in [(torch.float64, 1e-12), (torch.float32, 1e-5)]:
        A = Ainv.to(dt)
        y = torch.empty(n, dtype=dt, device="cuda")
        call("pmg_dense_gemv", 0 if dt == torch.float64 else 1, n, A, dev(b, dt), y, stream())
        ref = host(A) @ host(dev(b, dt))
        np.testing.assert_allclose(host(y), ref, rtol=0, atol=tol * np.abs(ref).max())


def test_chebyshev_smoother(pg):
    """l1 diagonals (stencil and matrix-free), step coefficients and smoothing steps against the same
    recurrence in numpy; the spectrum of D_l1^-1 A lies in (0, 1] and the smoother contracts."""
    from pymoto_gb300._lib import call, stream
    g, K, op, rng = _setup(pg, (8, 6, 4), seed=11)
    A1 = op.galerkin()
    Ad = host(A1.to_dense())
    n = Ad.shape[0]
    l1 = np.abs(Ad).sum(axis=1)
    deg, ratio = 3, 10.0
    sm = pg.Chebyshev(degree=deg, ratio=ratio)
    sm.update(A1)
    np.testing.assert_allclose(host(sm.D), l1, rtol=1e-13)
    assert np.linalg.eigvals(Ad / l1[:, None]).real.max() <= 1 + 1e-12
    # matrix-free finest operator: element bound >= assembled row sums of |K|
    sm0 = pg.Chebyshev(degree=2)
    sm0.update(op)
    Kd = K.toarray()
    D0 = host(sm0.D)
    assert np.all(D0 >= np.abs(Kd).sum(axis=1) * (1 - 1e-12))
    assert np.linalg.eigvals(Kd / D0[:, None]).real.max() <= 1 + 1e-12
    hi, lo = 1.0, 1.0 / ratio
    theta, delta = (hi + lo) / 2, (hi - lo) / 2
    sigma = theta / delta
    rho = 1 / sigma
    coef = [0.0, 1 / theta]
    for _ in range(1, deg):
        rn = 1 / (2 * sigma - rho)
        coef += [rn * rho, 2 * rn / delta]
        rho = rn
    np.testing.assert_allclose(host(sm.coef), coef, rtol=1e-13)
    b = rng.standard_normal(n)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    dv, r = torch.empty_like(x), torch.empty_like(x)
    res = sm.smooth(A1, dev(b), x, dv, r, zero_start=True)     # fused stencil steps
    xr = np.zeros(n)
    dr = coef[1] * b / l1
    xr = xr + dr
    for j in range(1, deg):
        dr = coef[2 * j] * dr + coef[2 * j + 1] * (b - Ad @ xr) / l1
        xr = xr + dr
    np.testing.assert_allclose(host(res), xr, rtol=1e-11, atol=1e-12 * np.abs(xr).max())
    # fused steps of the FP32 matrix-free level-0 operator from a nonzero start, against FP64 numpy
    from pymoto_gb300._lib import F32
    op32 = op.astype(F32)
    sm32 = pg.Chebyshev(degree=3, ratio=ratio)
    sm32.update(op32)
    D32 = host(sm32.D)
    x0 = rng.standard_normal(K.shape[0]).astype(np.float32)
    b0 = rng.standard_normal(K.shape[0]).astype(np.float32)
    xs = dev(x0, torch.float32)
    res32 = sm32.smooth(op32, dev(b0, torch.float32), xs, torch.empty_like(xs), torch.empty_like(xs), zero_start=False)
    xr = x0.astype(np.float64)
    dr = np.zeros_like(xr)
    for j in range(3):
        rr = b0 - Kd @ xr
        dr = (coef[2 * j] * dr if j else 0.0) + coef[2 * j + 1] * rr / D32
        xr = xr + dr
    assert np.abs(host(res32) - xr).max() <= 1e-4 * np.abs(xr).max()
    # error propagator I - X A of the smoother: spectral radius < 1
    Mi = np.diag(1 / l1)
    E = np.eye(n)
    Dk = coef[1] * Mi
    Xk = Dk.copy()
    for j in range(1, deg):
        Dk = coef[2 * j] * Dk + coef[2 * j + 1] * Mi @ (E - Ad @ Xk)
        Xk = Xk + Dk
    assert np.abs(np.linalg.eigvals(E - Xk @ Ad)).max() < 1.0


def test_cholesky_reports_not_spd(pg):
    from pymoto_gb300._lib import call, stream
    A = torch.eye(40, dtype=torch.float64, device="cuda")
    A[17, 17] = -1.0
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    call("pmg_cholesky_factor", 40, A, 39, info, stream())
    assert int(info.item()) == 18


@pytest.mark.parametrize("n", [1, 1000, 1 << 20, 3_000_017])
def test_dot_reductions_deterministic(pg, n):
    from pymoto_gb300._lib import call, stream
    from pymoto_gb300.operators import Workspace
    rng = np.random.default_rng(n)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    ws = Workspace.get()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    call("pmg_dot2", 0, n, dev(a), dev(b), dev(a), dev(a), out, ws.reduce, stream())
    o1 = out.cpu().numpy().copy()
    call("pmg_dot2", 0, n, dev(a), dev(b), dev(a), dev(a), out, ws.reduce, stream())
    assert np.array_equal(o1, out.cpu().numpy())  # run-to-run bitwise reproducible
    assert abs(o1[0] - a @ b) <= 1e-12 * np.sqrt(n) * max(1.0, abs(a @ b))
    assert abs(o1[1] - a @ a) <= 1e-12 * (a @ a)
    out32 = torch.zeros(1, dtype=torch.float64, device="cuda")
    call("pmg_dot", 1, n, dev(a, torch.float32), dev(b, torch.float32), out32, ws.reduce, stream())
    ref32 = a.astype(np.float32).astype(np.float64) @ b.astype(np.float32).astype(np.float64)
    assert abs(out32.item() - ref32) <= 1e-10 * np.sqrt(n)


def test_filters_golden(pg, golden):
    g = golden("filters.npz")
    for tag in ["q4", "q4r3", "h8", "h8r15"]:
        s = [int(v) for v in g[f"{tag}_shape"]]
        shape = tuple(s + [0] * (3 - len(s)))
        d = pg.VoxelDomain(*shape)
        r = float(g[f"{tag}_r"])
        x, dy = dev(g[f"{tag}_x"]), dev(g[f"{tag}_dy"])
        df = pg.DensityFilter(d, radius=r)
        np.testing.assert_allclose(host(df(x)), g[f"{tag}_density_y"], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(host(df._sensitivity(dy)), g[f"{tag}_density_dx"], rtol=1e-12, atol=1e-14)
        fc = pg.FilterConv(d, radius=r)
        np.testing.assert_allclose(host(fc(x)), g[f"{tag}_conv_y"], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(host(fc._sensitivity(dy)), g[f"{tag}_conv_dx"], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("mode", ["edge", "wrap"])
def test_conv_filter_other_paddings_are_adjoint(pg, mode):
    d = pg.VoxelDomain(9, 6, 5)
    fc = pg.FilterConv(d, radius=2.5, xmin_bc=mode, ymax_bc=mode)
    rng = np.random.default_rng(5)
    x, y = rng.standard_normal(d.nel), rng.standard_normal(d.nel)
    fx = host(fc(dev(x)))
    fty = host(fc._sensitivity(dev(y)))
    assert abs(fx @ y - x @ fty) <= 1e-12 * np.abs(fx @ y)
    # forward equals the padded convolution of the oracle's index-map definition
    maps = fc._maps_host
    I, J, K = np.meshgrid(*maps, indexing="ij")
    g = O.Grid(9, 6, 5)
    xp = x[g.elem_number(I, J, K)]
    W = fc.weights
    ref = np.zeros((9, 6, 5))
    for a in range(W.shape[0]):
        for b in range(W.shape[1]):
            for c in range(W.shape[2]):
                ref += W[-1 - a, -1 - b, -1 - c] * xp[a:a + 9, b:b + 6, c:c + 5]
    I, J, K = np.meshgrid(np.arange(9), np.arange(6), np.arange(5), indexing="ij")
    yref = np.zeros(g.nel)
    yref[g.elem_number(I, J, K).ravel()] = ref.ravel()
    np.testing.assert_allclose(fx, yref, rtol=1e-13, atol=1e-14)


def test_simp_and_sensitivity(pg):
    rng = np.random.default_rng(6)
    for shape in [(6, 4, 0), (5, 4, 3)]:
        g, K, op, _ = _setup(pg, shape, seed=7)
        x = rng.uniform(0, 1, g.nel)
        simp = pg.SIMP(xmin=1e-9, penal=3.0)
        np.testing.assert_allclose(host(simp(dev(x))), O.simp(x), rtol=1e-15)
        dy = rng.standard_normal(g.nel)
        np.testing.assert_allclose(host(simp._sensitivity(dev(dy))), dy * O.simp_derivative(x), rtol=1e-14)
        u, v = rng.standard_normal(g.ndof), rng.standard_normal(g.ndof)
        bc = clamp_face_dofs(g)
        K0 = O.element_stiffness(g)
        ref = O.sensitivity_contract(g, K0, [u], [v], bc)
        from pymoto_gb300._lib import call, stream
        dx = torch.empty(g.nel, dtype=torch.float64, device="cuda")
        call("pmg_sens_contract", *shape, K0, op.bcmask, dev(u), dev(v), 1.0, 0, dx, stream())
        np.testing.assert_allclose(host(dx), ref, rtol=1e-12, atol=1e-13 * np.abs(ref).max())
        # mixed contraction: FP32 quadratic form on FP64-shifted element vectors; displacements on a large
        # offset (the shift removes it exactly), error relative to the largest sensitivity
        off = 1e3 * np.tile([1.0, -2.0, 0.5][:g.dim], g.nnodes)
        ref2 = O.sensitivity_contract(g, K0, [u + off], [v - off], bc)
        dxm = torch.empty(g.nel, dtype=torch.float64, device="cuda")
        call("pmg_sens_contract_mixed", *shape, K0, op.bcmask, dev(u + off), dev(v - off), 1.0, 0, dxm, stream())
        assert np.abs(host(dxm) - ref2).max() <= 2e-6 * np.abs(ref2).max()


def test_oc_update_matches_oracle(pg):
    from pymoto_gb300._lib import call, stream
    from pymoto_gb300.operators import Workspace
    rng = np.random.default_rng(8)
    for n in [1200, 200_000]:
        x = rng.uniform(0.01, 1.0, n)
        dg = -rng.uniform(0, 10, n)
        dg[::17] = 1e-3  # positive entries are clipped to zero
        xn = torch.empty(n, dtype=torch.float64, device="cuda")
        call("pmg_oc_update", n, dev(x), dev(dg), xn, 0.4, 0.2, 0.0, 1.0, 0.0, 1e5, 1e-4, Workspace.get().oc, stream())
        np.testing.assert_allclose(host(xn), O.oc_step(x, dg, 0.4, move=0.2), rtol=1e-13, atol=1e-15)


def test_bad_arguments_are_rejected(pg):
    from pymoto_gb300._lib import PMGError, call, stream
    with pytest.raises(PMGError):
        call("pmg_restrict", 0, 5, 4, 0, None, None, stream())
    with pytest.raises(PMGError):
        call("pmg_ebe_apply", 7, 0, 4, 4, 0, None, None, None, 1.0, None, None, None, 0.0, None, None, stream())
