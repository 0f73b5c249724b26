"""FilterConv with constant-value padding and DensityFilter with `nonpadding`, against pyMOTO's own modules.

CPU: the host side (padded index maps with skipped positions, the constant field, the inverse maps of the
adjoint) evaluated by a numpy restatement of what the conv kernels compute.  GPU: the modules themselves."""
import numpy as np
import pytest
import torch

CONST_CASES = ["c3", "c2", "c3b"]
BCS = {"c3": dict(xmin_bc=0.0, xmax_bc=1.0, ymin_bc="edge", ymax_bc="wrap", zmin_bc=0.5, zmax_bc="symmetric"),
       "c2": dict(xmin_bc=1.0, xmax_bc="wrap", ymin_bc=0.0, ymax_bc=0.25),
       "c3b": dict(xmin_bc="wrap", xmax_bc="wrap", ymin_bc=0.0, ymax_bc=0.0, zmin_bc=1.0, zmax_bc=0.0)}


def _emulate(fc, x, d):
    """What conv_filter_kernel + the constant field and conv_filter_adjoint_kernel compute, in numpy."""
    g = fc.grid
    nx, ny, nz = g.nelx, g.nely, max(g.nelz, 1)
    kx, ky, kz = fc.weights.shape
    mx, my, mz = fc._maps_host
    elem = lambda i, j, k: (k * ny + j) * nx + i  # noqa: E731
    y = np.zeros(nx * ny * nz)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                acc = 0.0
                for c in range(kz):
                    kk = mz[k + kz - 1 - c]
                    for b in range(ky):
                        jj = my[j + ky - 1 - b]
                        for a in range(kx):
                            ii = mx[i + kx - 1 - a]
                            if kk < 0 or jj < 0 or ii < 0:
                                continue
                            acc += fc.weights[a, b, c] * x[elem(ii, jj, kk)]
                y[elem(i, j, k)] = acc
    if fc._const_host is not None:
        y = y + fc._const_host
    dx = np.zeros_like(y)
    inv = [fc._inverse_map(m, n) for m, n in zip(fc._maps_host, (nx, ny, nz))]
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                acc = 0.0
                for Pz in inv[2][1][inv[2][0][k]:inv[2][0][k + 1]]:
                    for Py in inv[1][1][inv[1][0][j]:inv[1][0][j + 1]]:
                        for Px in inv[0][1][inv[0][0][i]:inv[0][0][i + 1]]:
                            for c in range(kz):
                                oz = Pz - (kz - 1) + c
                                if not 0 <= oz < nz:
                                    continue
                                for b in range(ky):
                                    oy = Py - (ky - 1) + b
                                    if not 0 <= oy < ny:
                                        continue
                                    for a in range(kx):
                                        ox = Px - (kx - 1) + a
                                        if 0 <= ox < nx:
                                            acc += fc.weights[a, b, c] * d[elem(ox, oy, oz)]
                dx[elem(i, j, k)] = acc
    return y, dx


@pytest.mark.parametrize("tag", CONST_CASES)
def test_constant_padding_host_side_matches_pymoto(tag, golden):
    import pymoto_gb300 as pg
    g = golden("filter_variants.npz")
    d = pg.VoxelDomain(*[int(v) for v in g[f"{tag}_shape"]])
    fc = pg.FilterConv(d, radius=float(g[f"{tag}_r"]), **BCS[tag])
    y, dx = _emulate(fc, g[f"{tag}_x"], g[f"{tag}_dy"])
    np.testing.assert_allclose(y, g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(dx, g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


OVERRIDES = {"ov2": ({}, [((slice(0, 3), slice(2, 5), 0), 1.0), ((np.array([6, 7]), np.array([1, 1]), 0), 0.0)]),
             "ov3": (dict(ymax_bc=0.3), [((slice(None), 0, slice(1, 3)), 0.7), ((2, slice(None), 3), 0.0)])}


def _override_filter(tag, golden):
    import pymoto_gb300 as pg
    g = golden("filter_variants.npz")
    d = pg.VoxelDomain(*[int(v) for v in g[f"{tag}_shape"]])
    bcs, ovs = OVERRIDES[tag]
    fc = pg.FilterConv(d, radius=float(g[f"{tag}_r"]), **bcs)
    for idx, val in ovs:
        fc.override_values(idx, val)
    return fc, g


@pytest.mark.parametrize("tag", list(OVERRIDES))
def test_override_values_host_side_matches_pymoto(tag, golden):
    """y = F(x) + F0(1_S (v - x)) and dx = F^T dy - 1_S F0^T dy with the kernels' emulation."""
    fc, g = _override_filter(tag, golden)
    x, dy = g[f"{tag}_x"], g[f"{tag}_dy"]
    S = np.array(sorted(fc._overrides))
    v = np.array([fc._overrides[i] for i in S])
    d = np.zeros_like(x)
    d[S] = v - x[S]
    y, dx = _emulate(fc, x, dy)
    y0, t0 = _emulate(fc._fzero, d, dy)
    dx[S] -= t0[S]
    np.testing.assert_allclose(y + y0, g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(dx, g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(OVERRIDES))
def test_override_values_on_device(tag, golden):
    fc, g = _override_filter(tag, golden)
    y = fc(torch.from_numpy(g[f"{tag}_x"]).cuda())
    np.testing.assert_allclose(y.cpu().numpy(), g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    dx = fc._sensitivity(torch.from_numpy(g[f"{tag}_dy"]).cuda())
    np.testing.assert_allclose(dx.cpu().numpy(), g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("tag", ["np2", "np3"])
def test_oracle_nonpadding_matches_pymoto(tag, golden):
    import oracle as O
    g = golden("filter_variants.npz")
    grid = O.Grid(*[int(v) for v in g[f"{tag}_shape"]])
    H, s = O.density_filter_matrix(grid, float(g[f"{tag}_r"]))
    s = O.density_filter_nonpadding(s, g[f"{tag}_nonpad"])
    np.testing.assert_allclose(O.density_filter(H, s, g[f"{tag}_x"]), g[f"{tag}_y"], rtol=1e-13)
    np.testing.assert_allclose(O.density_filter_T(H, s, g[f"{tag}_dy"]), g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


def test_constant_zero_sides_need_no_field():
    import pymoto_gb300 as pg
    fc = pg.FilterConv(pg.VoxelDomain(6, 4), radius=1.5, xmin_bc=0.0, xmax_bc=0)
    assert fc._const_host is None and fc._maps_host[0][0] == -1 and fc._maps_host[0][-1] == -1


@pytest.mark.gpu
@pytest.mark.parametrize("tag", CONST_CASES)
def test_constant_padding_on_device(tag, golden):
    import pymoto_gb300 as pg
    g = golden("filter_variants.npz")
    d = pg.VoxelDomain(*[int(v) for v in g[f"{tag}_shape"]])
    fc = pg.FilterConv(d, radius=float(g[f"{tag}_r"]), **BCS[tag])
    x = torch.from_numpy(g[f"{tag}_x"]).cuda()
    np.testing.assert_allclose(fc(x).cpu().numpy(), g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    dy = torch.from_numpy(g[f"{tag}_dy"]).cuda()
    np.testing.assert_allclose(fc._sensitivity(dy).cpu().numpy(), g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["np2", "np3"])
def test_density_filter_nonpadding_on_device(tag, golden):
    import pymoto_gb300 as pg
    g = golden("filter_variants.npz")
    d = pg.VoxelDomain(*[int(v) for v in g[f"{tag}_shape"]])
    df = pg.DensityFilter(d, radius=float(g[f"{tag}_r"]), nonpadding=g[f"{tag}_nonpad"])
    x = torch.from_numpy(g[f"{tag}_x"]).cuda()
    np.testing.assert_allclose(df(x).cpu().numpy(), g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    dy = torch.from_numpy(g[f"{tag}_dy"]).cuda()
    np.testing.assert_allclose(df._sensitivity(dy).cpu().numpy(), g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


PADDED = {"po3": (dict(xmin_bc=0, xmax_bc="symmetric", ymin_bc=0, ymax_bc=0, zmin_bc=0, zmax_bc=0),
                  [(tuple(np.meshgrid(np.arange(2), 2 + np.arange(2, 4), 2 + np.arange(1, 4))), 1.0),
                   ((slice(10, 12), slice(3, 6), slice(2, 5)), 0.3),
                   ((np.array([3, 4]), np.array([4, 4]), np.array([3, 3])), 0.9),
                   ((slice(0, 1), slice(4, 5), slice(3, 4)), 0.2)]),
          "po2": (dict(xmin_bc="wrap", xmax_bc="wrap", ymin_bc="edge", ymax_bc=0.25),
                  [((slice(0, 2), slice(0, 2), 0), 0.6),
                   ((slice(None), 8, 0), 1.0),
                   ((np.array([10, 5]), np.array([3, 0]), np.array([0, 0])), np.array([0.4, 0.7]))])}


def _padded_filter(tag, golden):
    import pymoto_gb300 as pg
    g = golden("filter_variants.npz")
    d = pg.VoxelDomain(*[int(v) for v in g[f"{tag}_shape"]])
    bcs, povs = PADDED[tag]
    fc = pg.FilterConv(d, radius=float(g[f"{tag}_r"]), **bcs)
    for idx, val in povs:
        fc.override_padded_values(idx, val)
    return fc, g


@pytest.mark.parametrize("tag", list(PADDED))
def test_padded_overrides_host_side_matches_pymoto(tag, golden):
    """Kernel emulation + the ring terms (the module's own torch helper on CPU tensors) + the in-domain
    overrides reproduce pyMOTO's FilterConv with override_padded_values, forward and adjoint."""
    fc, g = _padded_filter(tag, golden)
    assert fc._padded and fc._overrides      # both kinds of position are exercised
    x, dy = g[f"{tag}_x"], g[f"{tag}_dy"]
    y, dx = _emulate(fc, x, dy)
    data = fc._padded_data(torch.device("cpu"))
    y = fc._padded_terms(torch.from_numpy(y), torch.from_numpy(x), data, False).numpy()
    dx = fc._padded_terms(torch.from_numpy(dx), torch.from_numpy(dy), data, True).numpy()
    S = np.array(sorted(fc._overrides))
    v = np.array([fc._overrides[i] for i in S])
    d = np.zeros_like(x)
    d[S] = v - x[S]
    y0, t0 = _emulate(fc._fzero, d, dy)
    dx[S] -= t0[S]
    np.testing.assert_allclose(y + y0, g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(dx, g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("tag", list(PADDED))
def test_padded_vector_and_domain_match_pymoto(tag, golden):
    fc, g = _padded_filter(tag, golden)
    np.testing.assert_array_equal(fc.get_padded_vector(g[f"{tag}_x"]), g[f"{tag}_xpad"])
    t = fc.get_padded_vector(torch.from_numpy(g[f"{tag}_x"]))
    np.testing.assert_array_equal(t.numpy(), g[f"{tag}_xpad"])
    pd = fc.padded_domain
    shape = g[f"{tag}_xpad"].shape
    assert (pd.nelx, pd.nely, max(pd.nelz, 1)) == shape


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(PADDED))
def test_padded_overrides_on_device(tag, golden):
    fc, g = _padded_filter(tag, golden)
    y = fc(torch.from_numpy(g[f"{tag}_x"]).cuda())
    np.testing.assert_allclose(y.cpu().numpy(), g[f"{tag}_y"], rtol=1e-13, atol=1e-15)
    dx = fc._sensitivity(torch.from_numpy(g[f"{tag}_dy"]).cuda())
    np.testing.assert_allclose(dx.cpu().numpy(), g[f"{tag}_dx"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("shape,r,nonpad", [((7, 5), 1.5, None), ((6, 5, 4), 2.0, None), ((10, 6), 2.5, "third")])
def test_density_filter_matrix_matches_the_oracle(shape, r, nonpad):
    """DensityFilter.H / .Hs (host, for code that reads them) equal the oracle's pyMOTO restatement."""
    import oracle as O
    import pymoto_gb300 as pg
    d = pg.VoxelDomain(*shape)
    npd = None if nonpad is None else np.arange(0, d.nel, 3)
    df = pg.DensityFilter(d, radius=r, nonpadding=npd)
    H, s = O.density_filter_matrix(O.Grid(*shape), r)
    if npd is not None:
        s = O.density_filter_nonpadding(s, npd)
    np.testing.assert_allclose(df.H.toarray(), H.toarray(), rtol=0, atol=1e-15)
    np.testing.assert_allclose(np.asarray(df.Hs).ravel(), np.asarray(s).ravel(), rtol=1e-15)


def test_new_radius_refreshes_the_derived_data():
    """set_filter_radius after construction (same kernel size) gives the state a fresh filter would have."""
    import pymoto_gb300 as pg
    d = pg.VoxelDomain(7, 5, 4)
    bcs = dict(xmin_bc=0.5, ymax_bc=1.0)
    a = pg.FilterConv(d, radius=2.5, **bcs)
    a.override_values((slice(0, 2), 1, 1), 0.3)
    a.set_filter_radius(2.8)
    b = pg.FilterConv(d, radius=2.8, **bcs)
    np.testing.assert_array_equal(a.weights, b.weights)
    np.testing.assert_array_equal(a._const_host, b._const_host)
    np.testing.assert_array_equal(a._fzero.weights, b.weights)
    assert a._dev is None and a._pad_dev is None
    with pytest.raises(ValueError):
        a.set_filter_radius(3.5)
