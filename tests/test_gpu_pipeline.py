"""End-to-end parity of the GPU path against pyMOTO's golden vectors and the oracle (GPU)."""
import numpy as np
import pytest
import torch

import oracle as O
from conftest import clamp_face_dofs

pytestmark = pytest.mark.gpu


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def host(t):
    return t.double().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.fixture(scope="module")
def pg():
    import pymoto_gb300 as pg
    pg._lib.load()
    return pg


def _shape3(s):
    s = [int(v) for v in s]
    return tuple(s + [0] * (3 - len(s)))


def build_network(pg, shape, bc, f, filt, radius, levels, tol, plane="strain", mixed=False, w=0.6, steps=2,
                  state_kind="numpy", sens_precision="fp64"):
    d = pg.VoxelDomain(*shape)
    x0 = np.full(d.nel, 0.5)
    sx = pg.Signal("x", x0 if state_kind == "numpy" else dev(x0))
    with pg.Network() as fn:
        xf = (pg.DensityFilter(d, radius=radius) if filt == "density" else pg.FilterConv(d, radius=radius))(sx)
        xs = pg.MathExpression("1e-9 + (1-1e-9)*inp0^3")(xf)
        sK = pg.AssembleStiffness(d, bc=bc, plane=plane, sensitivity_precision=sens_precision)(xs)
        if levels > 0:
            mgs = pg.GeometricMultigrid.hierarchy(d, levels=levels, smoother_w=w, smooth_steps=steps,
                                                  precision="fp32" if mixed else None)
            if mixed:
                solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=tol)
            else:
                solver = pg.CG(preconditioner=mgs[0], tol=tol)
        else:
            solver = None
        su = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)(sK, f if state_kind == "numpy" else dev(f))
        sc = pg.EinSum("i,i->")(su, f if state_kind == "numpy" else dev(f))
    return d, sx, su, sc, fn


def run_design(fn, sx, sc, x, kind="numpy"):
    sx.state = x if kind == "numpy" else dev(x)
    fn.response()
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    return float(sc.state), host(sx.sensitivity)


def test_vcycle_matches_reference(pg, golden):
    g = golden("multigrid.npz")
    for tag in ["q4", "h8", "h8b"]:
        shape = _shape3(g[f"{tag}_shape"])
        d = pg.VoxelDomain(*shape)
        K = pg.AssembleStiffness(d, bc=g[f"{tag}_bc"])(dev(g[f"{tag}_x"]))
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
        mgs[0].update(K)
        z = host(mgs[0].solve(dev(g[f"{tag}_r"])))
        np.testing.assert_allclose(z, g[f"{tag}_z"], rtol=0, atol=1e-11 * np.abs(g[f"{tag}_z"]).max())


@pytest.mark.parametrize("name", ["h8_mg", "q4_mg", "h8_direct"])
@pytest.mark.parametrize("state_kind", ["numpy", "torch"])
def test_pipeline_fp64_matches_reference(pg, golden, name, state_kind):
    """FP64 path vs pyMOTO's own FP64 results: compliance and sensitivities to 1e-8 relative."""
    g = golden(f"pipeline_{name}.npz")
    shape = _shape3(g["shape"])
    levels = int(g["levels"])
    filt = "conv" if name == "h8_mg" else "density"
    plane = "stress" if name == "q4_mg" else "strain"
    d, sx, su, sc, fn = build_network(pg, shape, g["bc"], g["f"], filt, float(g["radius"]), levels,
                                      float(g["tol"]), plane=plane, state_kind=state_kind)
    for it in range(2):
        c, dx = run_design(fn, sx, sc, g[f"x{it}"], state_kind)
        assert abs(c - float(g[f"c{it}"])) <= 1e-8 * abs(c), (c, float(g[f"c{it}"]))
        u = host(su.state)
        np.testing.assert_allclose(u, g[f"u{it}"], rtol=0, atol=1e-8 * np.abs(u).max())
        np.testing.assert_allclose(dx, g[f"dx{it}"], rtol=0, atol=1e-8 * np.abs(dx).max())


@pytest.mark.parametrize("sens_precision", ["fp64", "mixed"])
def test_pipeline_mixed_matches_reference(pg, golden, sens_precision):
    """Mixed path (FP64 flexible CG around the FP32 multigrid preconditioner; FP32 sensitivity contraction
    of FP64-shifted element vectors for "mixed") vs pyMOTO's own FP64 results on the hex8 pipeline, with the
    solve driven to an FP64 relative residual of 1e-8: compliance, u and sensitivities to 1e-6 relative."""
    g = golden("pipeline_h8_mg.npz")
    shape = _shape3(g["shape"])
    d, sx, su, sc, fn = build_network(pg, shape, g["bc"], g["f"], "conv", float(g["radius"]), int(g["levels"]),
                                      1e-8, mixed=True, sens_precision=sens_precision)
    for it in range(2):
        c, dx = run_design(fn, sx, sc, g[f"x{it}"])
        assert abs(c - float(g[f"c{it}"])) <= 1e-6 * abs(c), (c, float(g[f"c{it}"]))
        u = host(su.state)
        np.testing.assert_allclose(u, g[f"u{it}"], rtol=0, atol=1e-6 * np.abs(u).max())
        np.testing.assert_allclose(dx, g[f"dx{it}"], rtol=0, atol=1e-6 * np.abs(dx).max())


def test_cg_iterations_match_reference_algorithm(pg):
    """Same algorithm, same iterates: the FP64 GPU CG needs the oracle's iteration count (on a field
    mild enough that rounding cannot shift the count)."""
    shape = (16, 8, 8)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    rng = np.random.default_rng(0)
    x = O.simp(rng.uniform(0.5, 1.0, g.nel))
    K = O.assemble(g, O.element_stiffness(g), x, bc)
    hier = O.build_hierarchy(g, K, 3, w=0.6, smooth_steps=2)
    fr = f.copy()
    fr[bc] = 0
    u_ref, its_ref, _ = O.cg_solve(K, fr, lambda r: O.vcycle(hier[0], r), tol=1e-8)
    d = pg.VoxelDomain(*shape)
    Kop = pg.AssembleStiffness(d, bc=bc)(dev(x))
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)
    cg = pg.CG(preconditioner=mgs[0], tol=1e-8)
    cg.update(Kop)
    u = host(cg.solve(dev(fr)))
    assert abs((cg.iterations - 1) - its_ref) <= 0
    np.testing.assert_allclose(u, u_ref, rtol=0, atol=1e-9 * np.abs(u_ref).max())


def _cantilever_rhs(g):
    f = np.zeros(g.ndof)
    tip = g.node_number(g.nelx, g.nely // 2, g.nelz // 2)
    f[g.dim * tip + 1] = -1.0
    return f


@pytest.mark.parametrize("shape", [(32, 16, 16), (64, 32, 0)])
def test_mixed_precision_reaches_fp64_residual(pg, shape):
    """Mixed FP32/FP64 solve of the pipeline's stiffness (filtered random densities, r = 2.5, SIMP p = 3):
    true FP64 relative residual <= 1e-6 and compliance within 1e-6 of the oracle's FP64 solution."""
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = _cantilever_rhs(g)
    rng = np.random.default_rng(1)
    x = O.simp(O.conv_filter(g, O.conv_filter_weights(g, 2.5), rng.uniform(1e-3, 1.0, g.nel)))
    K = O.assemble(g, O.element_stiffness(g), x, bc)
    fr = f.copy()
    fr[bc] = 0
    u_ref = O.direct_solve(K, fr) if g.ndof < 60000 else O.cg_solve(K, fr, tol=1e-12)[0]
    c_ref = fr @ u_ref
    d = pg.VoxelDomain(*shape)
    Kop = pg.AssembleStiffness(d, bc=bc)(dev(x))
    mgs = pg.GeometricMultigrid.hierarchy(d, smoother_w=0.6, smooth_steps=2, precision="fp32")
    solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-6)
    solver.update(Kop)
    u = solver.solve(dev(fr))
    res = pg.LinearSolver.residual(Kop, u, dev(fr))
    assert res <= 1e-6
    c = float(fr @ host(u))
    assert abs(c - c_ref) <= 1e-6 * abs(c_ref)
    assert not solver.fell_back


def test_lagged_coarse_inverse_is_promoted(pg):
    """coarse_lag: the first update factorises synchronously; a later update keeps the previous coarse inverse
    active until its own factorisation finishes, the solver promotes the new one mid-solve, and the solve
    reaches the FP64 tolerance.  After the solve the active inverse is that of the current coarse matrix."""
    shape = (32, 16, 16)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = _cantilever_rhs(g)
    f[bc] = 0
    rng = np.random.default_rng(4)
    w = O.conv_filter_weights(g, 2.5)
    d = pg.VoxelDomain(*shape)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=4, smooth_steps=1, coarse_smooth_steps=3, precision="fp32",
                                          smoother="chebyshev", coarse_lag=True)
    solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-6, inner_iters=3)
    coarse = mgs[-1].inner_level
    assert isinstance(coarse, pg.DenseCholesky) and coarse.lag
    for it in range(3):
        x = O.simp(O.conv_filter(g, w, rng.uniform(1e-3, 1.0, g.nel)))
        Kop = pg.AssembleStiffness(d, bc=bc)(dev(x))
        solver.update(Kop)
        u = solver.solve(dev(f))
        assert pg.LinearSolver.residual(Kop, u, dev(f)) <= 1e-6
        torch.cuda.synchronize()
        assert coarse.promote_if_ready()
        fresh = pg.DenseCholesky()
        fresh.update(mgs[-1]._Ac)
        assert torch.equal(coarse.Ainv32, fresh.Ainv32)


def test_mixed_precision_falls_back_on_extreme_contrast(pg):
    """Unfiltered SIMP noise (element-to-element contrast up to 1e9): the FP32 preconditioner stalls, the
    solver switches to the FP64 hierarchy and still reaches the FP64 residual tolerance."""
    shape = (16, 8, 8)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = _cantilever_rhs(g)
    f[bc] = 0
    x = O.simp(np.random.default_rng(1).uniform(1e-3, 1.0, g.nel))
    d = pg.VoxelDomain(*shape)
    Kop = pg.AssembleStiffness(d, bc=bc)(dev(x))
    mgs = pg.GeometricMultigrid.hierarchy(d, smoother_w=0.6, smooth_steps=2, precision="fp32")
    solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-6, maxit=400, stall_window=20)
    solver.update(Kop)
    u = solver.solve(dev(f))
    assert pg.LinearSolver.residual(Kop, u, dev(f)) <= 1e-6


def test_oc_trajectory_matches_reference(pg, golden):
    """60x20 half-MBB, DensityFilter r=1.5, OC move 0.2: 50 design iterations on the device."""
    g = golden("oc_mbb.npz")
    d = pg.VoxelDomain(60, 20)
    sx = pg.Signal("x", dev(np.full(d.nel, 0.5)))
    with pg.Network() as fn:
        xf = pg.DensityFilter(d, radius=1.5)(sx)
        xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
        K = pg.AssembleStiffness(d, bc=g["bc"], plane="stress")(xs)
        u = pg.LinSolve(hermitian=True, symmetric=True)(K, dev(g["f"]))
        c = pg.EinSum("i,i->")(u, dev(g["f"]))
    oc = pg.OC(sx, c, fn, move=0.2, verbosity=0)
    x_eval = None
    for _ in range(50):
        x_eval = host(sx.state)
        oc.step()
    np.testing.assert_allclose(oc.history, g["c_hist"], rtol=1e-6)
    np.testing.assert_allclose(x_eval, g["x_final"], atol=1e-5)


def test_sensitivity_central_differences(pg):
    """Adjoint sensitivities vs central finite differences on 64 seeded elements.  h = 1e-4 x keeps the
    solver's rounding (~1e-14 c) / h below the rtol while the O(h^2) truncation stays ~1e-8."""
    shape = (16, 8, 8)
    d = pg.VoxelDomain(*shape)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    rng = np.random.default_rng(2)
    x = rng.uniform(0.1, 1.0, g.nel)
    d_, sx, su, sc, fn = build_network(pg, shape, bc, f, "conv", 2.5, 3, 1e-12)
    c0, dx = run_design(fn, sx, sc, x)
    els = rng.choice(g.nel, 64, replace=False)
    fd = []
    for e in els:
        h = 1e-4 * x[e]
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        sx.state = xp
        fn.response()
        cp = float(sc.state)
        sx.state = xm
        fn.response()
        cm = float(sc.state)
        fd.append((cp - cm) / (2 * h))
    fd = np.array(fd)
    np.testing.assert_allclose(dx[els], fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


def test_autograd_compliance_function(pg):
    """torch.autograd through the compliance path: the backward of pg.ComplianceObjective (the adjoint
    kernels behind a torch.autograd.Function) equals the module network's sensitivity() and central finite
    differences, and composes with ordinary torch operations."""
    shape = (16, 8, 8)
    d = pg.VoxelDomain(*shape)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    rng = np.random.default_rng(5)
    x = rng.uniform(0.1, 1.0, g.nel)
    solver = pg.CG(preconditioner=pg.GeometricMultigrid.hierarchy(d, levels=3, smoother_w=0.6, smooth_steps=2)[0],
                   tol=1e-12)
    obj = pg.ComplianceObjective(d, bc, f, radius=2.5, penal=3.0, xmin=1e-9, solver=solver)
    xt = dev(x).requires_grad_(True)
    c = obj(xt)
    c.backward()
    grad = host(xt.grad)
    c = c.detach()
    # the same modules driven by the graph runtime
    _, sx, _, sc, fn = build_network(pg, shape, bc, f, "conv", 2.5, 3, 1e-12)
    c_ref, dx_ref = run_design(fn, sx, sc, x)
    assert abs(float(c) - c_ref) <= 1e-10 * abs(c_ref)
    np.testing.assert_allclose(grad, dx_ref, rtol=1e-7, atol=1e-9 * np.abs(dx_ref).max())
    # central differences on 16 elements
    els = rng.choice(g.nel, 16, replace=False)
    for e in els:
        h = 1e-4 * x[e]
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (obj(dev(xp)).item() - obj(dev(xm)).item()) / (2 * h)
        assert abs(grad[e] - fd) <= 1e-5 * abs(fd) + 1e-6 * np.abs(grad).max()
    # chain rule with torch operations around it
    xt2 = dev(x).requires_grad_(True)
    loss = obj(xt2) ** 2 + xt2.sum()
    loss.backward()
    np.testing.assert_allclose(host(xt2.grad), 2 * float(c) * grad + 1.0, rtol=1e-9, atol=1e-12)
