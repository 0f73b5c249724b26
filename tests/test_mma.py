"""MMA: the oracle against pyMOTO's own MMA steps (CPU), the C ABI's argument checks (CPU), and the device update
against pyMOTO and the oracle (GPU)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle.mma import MMAOracle

CASES = [("v2007", "MMA2007"), ("v1987", "MMA1987"), ("unc", "MMA2007")]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("tag,version", CASES)
def test_oracle_reproduces_pymoto_mma_steps(tag, version, golden):
    g = golden("mma_mbb.npz")
    X, G, DG = g[f"{tag}_x"], g[f"{tag}_g"], g[f"{tag}_dg"]
    o = MMAOracle(X.shape[1], G.shape[1], move=0.2, mmaversion=version)
    for k in range(X.shape[0]):
        xn = o.step(X[k], G[k], DG[k])
        # same numpy operations in the same order: equal up to the last bit on one machine; 1e-13 across
        # BLAS builds (the m-term dot products)
        np.testing.assert_allclose(xn, g[f"{tag}_xnew"][k], rtol=0, atol=1e-13)
        np.testing.assert_allclose(o.low, g[f"{tag}_low"][k], rtol=1e-15)
        np.testing.assert_allclose(o.offset, g[f"{tag}_offset"][k], rtol=1e-15)
        np.testing.assert_allclose(o.gest, g[f"{tag}_gest"][k], rtol=1e-12, atol=1e-13)
        assert abs(o.dk - g[f"{tag}_dk"][k]) <= 1e-12 * abs(g[f"{tag}_dk"][k])


def test_params_struct_layout_and_argument_checks():
    from pymoto_gb300._lib import PMGError, call
    from pymoto_gb300.mma import _Params
    # 6 ints, 7 doubles, rho[5], a[4], c[4], d[4] (include/pymoto_gb300.h)
    assert ctypes.sizeof(_Params) == 24 + 7 * 8 + 5 * 8 + 3 * 4 * 8
    assert call("pmg_mma_scratch_bytes", 100, 5) == 0 and call("pmg_mma_scratch_bytes", 0, 1) == 0
    assert call("pmg_mma_scratch_bytes", 1000, 2) > (8 + 6 + 2) * 1000 * 8
    p = _Params()
    p.version, p.m, p.maxit, p.epsimin = 1, 5, 400, 1e-9      # m above PMG_MMA_MAX_M: rejected before a launch
    with pytest.raises(PMGError) as e:
        call("pmg_mma_update", 10, ctypes.addressof(p), *([1] * 15))
    assert e.value.status == 1
    p.m, p.epsimin = 1, 0.0                                     # epsilon must be positive
    with pytest.raises(PMGError):
        call("pmg_mma_update", 10, ctypes.addressof(p), *([1] * 15))


def test_scaling_module_formulas():
    import pymoto_gb300 as pg
    s = pg.Scaling(scaling=100.0)
    assert s(4.0) == pytest.approx(100.0) and s(2.0) == pytest.approx(50.0)
    assert s._sensitivity(1.0) == pytest.approx(25.0)
    s = pg.Scaling(scaling=5.0, maxval=150.0)
    assert s(160.0) == pytest.approx(5.0 * 10.0 / 150.0)
    assert s._sensitivity(1.0) == pytest.approx(5.0 / 150.0)
    s = pg.Scaling(scaling=2.0, minval=-4.0)
    assert s(-6.0) == pytest.approx(2.0 * 2.0 / 4.0) and s._sensitivity(1.0) == pytest.approx(-0.5)


# ---- device ------------------------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("tag,version", CASES)
def test_device_update_matches_pymoto_steps(tag, version, exact, golden):
    from pymoto_gb300.mma import MMAUpdate
    g = golden("mma_mbb.npz")
    X, G, DG = g[f"{tag}_x"], g[f"{tag}_g"], g[f"{tag}_dg"]
    up = MMAUpdate(X.shape[1], G.shape[1], 0.0, 1.0, move=0.2, mmaversion=version, exact=exact)
    o = MMAOracle(X.shape[1], G.shape[1], move=0.2, mmaversion=version)
    for k in range(X.shape[0]):
        xn = up.step(dev(X[k]), dev(G[k]), dev(DG[k])).cpu().numpy()
        o.step(X[k], G[k], DG[k])
        # exact: element-wise values round as numpy's (no FMA contraction); fast: within a few ulp.  The sums over
        # elements are in another order, so the interior-point iterates differ in the last bits: x to 1e-8 (the
        # subproblem's tolerance is epsimin sqrt(n+m) ~ 2e-9); asymptotes and offsets exactly
        np.testing.assert_allclose(xn, g[f"{tag}_xnew"][k], rtol=0, atol=1e-8)
        np.testing.assert_allclose(up.low.cpu().numpy(), g[f"{tag}_low"][k], rtol=1e-15)
        np.testing.assert_allclose(up.upp.cpu().numpy(), g[f"{tag}_upp"][k], rtol=1e-15)
        np.testing.assert_allclose(up.offset.cpu().numpy(), g[f"{tag}_offset"][k], rtol=1e-15)
        np.testing.assert_allclose(up.gest, g[f"{tag}_gest"][k], rtol=1e-7, atol=1e-8)
        assert abs(up.dk - g[f"{tag}_dk"][k]) <= 1e-6 * abs(g[f"{tag}_dk"][k])
        st = up.stats
        assert st["outer"] == o.stats["outer"]
        assert abs(st["newton"] - o.stats["newton"]) <= 2


@pytest.mark.gpu
@pytest.mark.parametrize("m", [2, 3, 4])
def test_device_update_several_constraints_vs_oracle(m):
    """Three chained steps (the third adapts the asymptotes) of a 20,000-variable problem with m constraints."""
    from pymoto_gb300.mma import MMAUpdate
    rng = np.random.default_rng(300 + m)
    n = 20000
    x = rng.uniform(0.05, 0.95, n)
    up = MMAUpdate(n, m + 1, 0.0, 1.0, move=0.1, mmaversion="MMA2007")
    o = MMAOracle(n, m + 1, move=0.1, mmaversion="MMA2007")
    for k in range(3):
        g = np.concatenate([[1.0 + 0.1 * k], rng.uniform(-0.2, 0.1, m)])
        dg = np.vstack([-rng.uniform(0.0, 2.0, n) / n, rng.standard_normal((m, n)) / n])
        xo = o.step(x, g, dg)
        xd = up.step(dev(x), dev(g), dev(dg)).cpu().numpy()
        np.testing.assert_allclose(xd, xo, rtol=0, atol=1e-8)
        np.testing.assert_allclose(up.gest, o.gest, rtol=1e-7, atol=1e-8)
        x = xo


@pytest.mark.gpu
@pytest.mark.parametrize("tag,version", [("v2007", "MMA2007"), ("gcmma", "GCMMA")])
def test_mma_optimizer_on_the_device_network(tag, version, golden):
    """pyMOTO's MMA run (30x10 half-MBB, DensityFilter r=1.5, objective Scaling(100) of the compliance, volume
    constraint 10 (sum(xf)/nel - 0.5)) with every module, the sensitivities and the update on the device.  The
    constraint is built as Scaling(5, maxval=nel/2) of the volume, the same function of x."""
    import pymoto_gb300 as pg
    g = golden("mma_mbb.npz")
    d = pg.VoxelDomain(30, 10)
    f = dev(g[f"{tag}_f"])
    sx = pg.Signal("x", dev(np.full(d.nel, 0.5)))
    with pg.Network() as fn:
        xf = pg.DensityFilter(d, radius=1.5)(sx)
        xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
        K = pg.AssembleStiffness(d, bc=g[f"{tag}_bc"], plane="stress")(xs)
        u = pg.LinSolve(hermitian=True, symmetric=True)(K, f)
        c = pg.EinSum("i,i->")(u, f)
        g0 = pg.Scaling(scaling=100.0)(c)
        vol = pg.EinSum("i->")(xf)
        g1 = pg.Scaling(scaling=5.0, maxval=0.5 * d.nel)(vol)
    mma = pg.MMA(sx, [g0, g1], fn, move=0.2, verbosity=0, mmaversion=version)
    xval = mma.x
    for k in range(g[f"{tag}_x"].shape[0]):
        xnew, gk, _ = mma.step(x=xval)
        np.testing.assert_allclose(xval.cpu().numpy(), g[f"{tag}_x"][k], rtol=0, atol=1e-6)
        np.testing.assert_allclose(gk.cpu().numpy(), g[f"{tag}_g"][k], rtol=1e-6, atol=1e-8)
        np.testing.assert_allclose(xnew.cpu().numpy(), g[f"{tag}_xnew"][k], rtol=0, atol=1e-5)
        xval = xnew
