"""Springs to ground: AssembleStiffness(add_constant=...) (pymoto/modules/assembly.py:294-295).

The constant is added after the Dirichlet rows are set, so a constrained dof holds bcdiagval + its spring.  The
matrix-free operators take a constant diagonal: the FP64 stencils and the FP32 matrix-free product of level 0
add it exactly, the coarse multigrid levels its restriction R^T c (lumped), which keeps them nonsingular when the
springs are the only supports.  Fixtures written by pyMOTO (tests/golden/make_golden.py springs): a 2D
mechanism-like case, a 3D cantilever with springs (one on a Dirichlet dof) and a 3D case supported by springs
only.
"""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

import oracle as O

CASES = ["q4", "h8", "soft"]


def _shape(g, tag):
    return tuple(int(v) for v in g[f"{tag}_shape"])


def _oracle_matrix(g, tag):
    grid = O.Grid(*_shape(g, tag))
    K0 = O.element_stiffness(grid)
    bc = g[f"{tag}_bc"]
    K = O.assemble(grid, K0, g[f"{tag}_x"], bc if bc.size else None)
    n = grid.ndof
    C = sps.csr_matrix((g[f"{tag}_val"], (g[f"{tag}_idx"], g[f"{tag}_idx"])), shape=(n, n))
    return (K + C).tocsr()


@pytest.mark.parametrize("tag", CASES)
def test_oracle_with_springs_matches_pymoto(golden, tag):
    """The oracle's K + diag(c) and its direct solve reproduce pyMOTO's (CPU)."""
    g = golden("springs.npz")
    A = _oracle_matrix(g, tag)
    Ku = A @ g[f"{tag}_urand"]
    np.testing.assert_allclose(Ku, g[f"{tag}_Ku"], rtol=0, atol=1e-13 * np.abs(Ku).max())
    u = O.direct_solve(A, g[f"{tag}_f"])
    np.testing.assert_allclose(u, g[f"{tag}_u"], rtol=0, atol=1e-10 * np.abs(u).max())


def test_non_diagonal_constant_is_rejected():
    import pymoto_gb300 as pg
    d = pg.VoxelDomain(4, 2)
    n = d.nnodes * 2
    C = sps.csr_matrix((np.ones(2), ([0, 1], [1, 0])), shape=(n, n))
    with pytest.raises(NotImplementedError):
        pg.AssembleStiffness(d, add_constant=C)
    pg.AssembleStiffness(d, add_constant=sps.identity(n))         # diagonal: accepted
    pg.AssembleStiffness(d, add_constant=np.ones(n))              # its diagonal as a vector: accepted


def _network(pg, g, tag, precision):
    shape = _shape(g, tag)
    d = pg.VoxelDomain(*shape)
    n = g[f"{tag}_f"].size
    C = sps.csc_matrix((g[f"{tag}_val"], (g[f"{tag}_idx"], g[f"{tag}_idx"])), shape=(n, n))
    bc = g[f"{tag}_bc"]
    sx = pg.Signal("x", torch.from_numpy(g[f"{tag}_x"]).cuda())
    f = torch.from_numpy(g[f"{tag}_f"]).cuda()
    with pg.Network() as fn:
        sK = pg.AssembleStiffness(d, bc=bc if bc.size else None, add_constant=C)(sx)
        levels = 2 if tag != "h8" else 3      # 12x6 and 6x4x4 halve once, 8x4x4 twice
        if precision == "mixed":
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=levels, smooth_steps=1, precision="fp32",
                                                  coarse_smooth_steps=[2] * (levels - 1), smoother="chebyshev")
            solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-10)
        else:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=levels, smoother_w=0.6, smooth_steps=2)
            solver = pg.CG(preconditioner=mgs[0], tol=1e-12, maxit=5000)
        su = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)(sK, f)
        sc = pg.EinSum("i,i->")(su, f)
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    return sK, su, sc, sx


@pytest.mark.gpu
@pytest.mark.parametrize("tag", CASES)
def test_operator_with_springs_matches_pymoto(golden, tag):
    """K u with the constant diagonal: FP64 stencil product to 1e-13, FP32 product to FP32 accuracy; the
    diagonal includes the springs."""
    import pymoto_gb300 as pg
    from pymoto_gb300._lib import F32
    g = golden("springs.npz")
    sK, _, _, _ = _network(pg, g, tag, "fp64")
    K = sK.state
    ur = torch.from_numpy(g[f"{tag}_urand"]).cuda()
    ref = g[f"{tag}_Ku"]
    y = K.matvec(ur).cpu().numpy()
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    y32 = K.astype(F32).matvec(ur.float()).double().cpu().numpy()
    assert np.abs(y32 - ref).max() <= 1e-5 * np.abs(ref).max()
    A = _oracle_matrix(g, tag)
    np.testing.assert_allclose(K.diagonal().cpu().numpy(), A.diagonal(), rtol=1e-14, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("tag", CASES)
def test_network_with_springs_matches_pymoto(golden, tag, precision):
    """Solution, compliance and sensitivities of the spring-supported networks against pyMOTO's (FP64 path to
    1e-8; the mixed path, solved to an FP64 residual of 1e-10, to 1e-7)."""
    import pymoto_gb300 as pg
    g = golden("springs.npz")
    _, su, sc, sx = _network(pg, g, tag, precision)
    tol = 1e-8 if precision == "fp64" else 1e-7
    u = su.state.cpu().numpy()
    np.testing.assert_allclose(u, g[f"{tag}_u"], rtol=0, atol=tol * np.abs(g[f"{tag}_u"]).max())
    assert abs(float(sc.state) - float(g[f"{tag}_c"])) <= tol * abs(float(g[f"{tag}_c"]))
    dx = sx.sensitivity.cpu().numpy()
    np.testing.assert_allclose(dx, g[f"{tag}_dx"], rtol=0, atol=tol * np.abs(g[f"{tag}_dx"]).max())
