"""Write the golden fixtures of tests/golden/ by running pyMOTO itself (v2.0.1).

Run where the pyMOTO sources are available: give their path with --reference PATH or in
$PYMOTO_REFERENCE; without either, a pyMOTO checkout named "reference" beside this repository is used.  matplotlib is not needed: a module stub stands in for it, because pyMOTO imports it
at module level for plotting only.  The fixtures are small .npz files; the tests never import pyMOTO.

    python tests/golden/make_golden.py --reference PATH          # every fixture
    python tests/golden/make_golden.py vti      # the VTI files only
    python tests/golden/make_golden.py mma      # the MMA steps only
    python tests/golden/make_golden.py scalars  # the ScalarToFile logs only
    python tests/golden/make_golden.py filters2 # the FilterConv / DensityFilter variants only
    python tests/golden/make_golden.py domain   # the VoxelDomain geometry helpers only
    python tests/golden/make_golden.py mass     # the AssembleMass matrices only
    python tests/golden/make_golden.py math     # the MathExpression cases only
    python tests/golden/make_golden.py overhang # the OverhangFilter cases only
    python tests/golden/make_golden.py poisson  # the AssemblePoisson cases only
    python tests/golden/make_golden.py poisson_mg  # multigrid on one-component (AssemblePoisson) matrices only
    python tests/golden/make_golden.py einsum   # the EinSum expressions only
    python tests/golden/make_golden.py springs  # AssembleStiffness add_constant (springs to ground) only
"""
import os
import sys
import types
import warnings

import numpy as np

def _default_reference():
    """$PYMOTO_REFERENCE, else a pyMOTO checkout named "reference" beside this repository (None if absent)."""
    env = os.environ.get("PYMOTO_REFERENCE")
    if env:
        return env
    sibling = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))))), "reference")
    return sibling if os.path.isdir(os.path.join(sibling, "pymoto")) else None


REF = _default_reference()
OUT = os.path.dirname(os.path.abspath(__file__))


def import_reference():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl
    for sub in ["patches", "path", "pyplot", "colors", "cm", "figure", "axes"]:
        m = types.ModuleType("matplotlib." + sub)
        sys.modules["matplotlib." + sub] = m
        setattr(mpl, sub, m)
    sys.modules["matplotlib.patches"].PathPatch = object
    sys.modules["matplotlib.path"].Path = object
    if not REF or not os.path.isdir(os.path.join(REF, "pymoto")):
        raise SystemExit("make_golden: give the pyMOTO sources with --reference PATH or $PYMOTO_REFERENCE")
    sys.path.insert(0, REF)
    import pymoto
    return pymoto


def clamp_face_dofs(d, dim):
    nodes = d.nodes[0, ...].flatten()
    return (nodes[:, None] * dim + np.arange(dim)).ravel()


def save(name, **arrs):
    np.savez_compressed(os.path.join(OUT, name), **arrs)
    print("wrote", name, sorted(arrs))


def maps_and_k0(pym):
    out = {}
    for tag, shp, units in [("q4", (6, 4), (1.0, 1.0, 1.0)), ("q4s", (5, 3), (0.5, 2.0, 0.3)),
                            ("h8", (4, 3, 2), (1.0, 1.0, 1.0)), ("h8s", (3, 2, 2), (0.1, 0.2, 0.3))]:
        d = pym.VoxelDomain(*shp, unitx=units[0], unity=units[1], unitz=units[2])
        out[f"{tag}_shape"] = np.array(shp)
        out[f"{tag}_units"] = np.array(units)
        out[f"{tag}_conn"] = d.conn
        out[f"{tag}_dofconn"] = d.get_dofconnectivity(d.dim)
        out[f"{tag}_K0"] = pym.AssembleStiffness(d).stiffness_element
        if d.dim == 2:
            out[f"{tag}_K0stress"] = pym.AssembleStiffness(d, plane="stress").stiffness_element
    save("maps_k0.npz", **out)


def assembly(pym):
    out = {}
    for tag, shp in [("q4", (6, 4)), ("h8", (4, 3, 2))]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(7)
        x = rng.uniform(0.05, 1.0, d.nel)
        bc = clamp_face_dofs(d, d.dim)
        K = pym.AssembleStiffness(d, bc=bc)(x).tocsr()
        K.eliminate_zeros()
        u = rng.standard_normal(K.shape[0])
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_x": x, f"{tag}_bc": bc, f"{tag}_data": K.data,
                    f"{tag}_indices": K.indices, f"{tag}_indptr": K.indptr, f"{tag}_u": u,
                    f"{tag}_Ku": K @ u})
    save("assembly.npz", **out)


def filters(pym):
    out = {}
    for tag, shp, r in [("q4", (10, 6), 1.5), ("q4r3", (9, 7), 3.0), ("h8", (8, 6, 4), 2.5), ("h8r15", (5, 4, 3), 1.5)]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(3)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        df = pym.DensityFilter(d, radius=r)
        fc = pym.FilterConv(d, radius=r)
        sx = pym.Signal("x", x)
        sy = fc(sx)
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_r": np.array(r), f"{tag}_x": x, f"{tag}_dy": dy,
                    f"{tag}_density_y": df(x), f"{tag}_density_dx": df._sensitivity(dy),
                    f"{tag}_conv_y": sy.state, f"{tag}_conv_dx": fc._sensitivity(dy),
                    f"{tag}_conv_w": fc.weights})
    save("filters.npz", **out)


def multigrid(pym):
    out = {}
    for tag, shp in [("q4", (8, 4)), ("h8", (4, 4, 4)), ("h8b", (8, 4, 4))]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(11)
        x = rng.uniform(1e-3, 1.0, d.nel) ** 3
        bc = clamp_face_dofs(d, d.dim)
        K = pym.AssembleStiffness(d, bc=bc)(x)
        mg1 = pym.solvers.GeometricMultigrid(d, smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2)
        mg2 = pym.solvers.GeometricMultigrid(mg1.sub_domain, smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2)
        mg1.inner_level = mg2
        mg1.update(K)
        R = mg1.R.tocoo()
        Ac = mg1.inner_level.A.tocsr()
        Ac.eliminate_zeros()
        r = rng.standard_normal(K.shape[0])
        r[bc] = 0.0
        z = mg1.solve(r)
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_x": x, f"{tag}_bc": bc,
                    f"{tag}_R_row": R.row, f"{tag}_R_col": R.col, f"{tag}_R_val": R.data,
                    f"{tag}_Ac_data": Ac.data, f"{tag}_Ac_indices": Ac.indices, f"{tag}_Ac_indptr": Ac.indptr,
                    f"{tag}_r": r, f"{tag}_z": z})
    save("multigrid.npz", **out)


def pipeline(pym, tag, shp, filt, radius, levels, tol, plane="strain"):
    d = pym.VoxelDomain(*shp)
    dim = d.dim
    bc = clamp_face_dofs(d, dim)
    f = np.zeros(d.nnodes * dim)
    if dim == 2:
        f[dim * d.get_nodenumber(shp[0], shp[1] // 2) + 1] = -1.0
    else:
        f[dim * d.get_nodenumber(shp[0], shp[1] // 2, shp[2] // 2) + 1] = -1.0
    rng = np.random.default_rng(5)
    x1 = rng.uniform(1e-3, 1.0, d.nel)
    x2 = np.clip(x1 + 0.05 * (rng.uniform(size=d.nel) - 0.5), 1e-3, 1.0)
    sx = pym.Signal("x", x1)
    with pym.Network() as fn:
        xf = (pym.DensityFilter(d, radius=radius) if filt == "density" else pym.FilterConv(d, radius=radius))(sx)
        xs = pym.MathExpression("1e-9 + (1-1e-9)*inp0^3")(xf)
        sK = pym.AssembleStiffness(d, bc=bc, plane=plane)(xs)
        if levels > 0:
            mgs = [pym.solvers.GeometricMultigrid(d, smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2)]
            while len(mgs) < levels - 1:
                mgs.append(pym.solvers.GeometricMultigrid(mgs[-1].sub_domain,
                                                          smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2))
                mgs[-2].inner_level = mgs[-1]
            solver = pym.solvers.CG(preconditioner=mgs[0], tol=tol)
        else:
            solver = None
        su = pym.LinSolve(hermitian=True, symmetric=True, solver=solver)(sK, f)
        sc = pym.EinSum("i,i->")(su, f)
    res = {"shape": np.array(shp), "bc": bc, "f": f, "radius": np.array(radius), "levels": np.array(levels),
           "tol": np.array(tol)}
    for it, x in enumerate([x1, x2]):
        sx.state = x
        fn.response()
        fn.reset()
        sc.sensitivity = 1.0
        fn.sensitivity()
        res.update({f"x{it}": x, f"u{it}": su.state.copy(), f"c{it}": np.array(sc.state),
                    f"dx{it}": sx.sensitivity.copy()})
    save(f"pipeline_{tag}.npz", **{k: v for k, v in res.items()})


def oc_mbb(pym):
    """60x20 half-MBB beam, DensityFilter r=1.5, plane stress, direct solve, OC move 0.2, 50 iterations."""
    d = pym.VoxelDomain(60, 20)
    left_x = 2 * d.nodes[0, :].flatten()
    br_y = 2 * d.get_nodenumber(60, 0) + 1
    bc = np.concatenate([left_x, [br_y]])
    f = np.zeros(d.nnodes * 2)
    f[2 * d.get_nodenumber(0, 20) + 1] = -1.0
    sx = pym.Signal("x", np.full(d.nel, 0.5))
    with pym.Network() as fn:
        xf = pym.DensityFilter(d, radius=1.5)(sx)
        xs = pym.MathExpression("1e-9 + (1-1e-9)*inp0^3")(xf)
        K = pym.AssembleStiffness(d, bc=bc, plane="stress")(xs)
        u = pym.LinSolve(hermitian=True, symmetric=True)(K, f)
        c = pym.EinSum("i,i->")(u, f)
    hist = [float(c.state)]  # the first response ran when the network was built
    orig = fn.response

    def resp():
        orig()
        hist.append(float(c.state))
    fn.response = resp
    oc = pym.OC(sx, c, fn, move=0.2, verbosity=0)
    oc.optimize(maxiter=50, tolx=0, tolf=0)
    save("oc_mbb.npz", bc=bc, f=f, c_hist=np.array(hist), x_final=sx.state.copy())


def mma_mbb(pym):
    """pyMOTO's MMA on a 30x10 half-MBB beam (DensityFilter r=1.5, plane stress, direct solve): objective
    Scaling(100) of the compliance, constraint 10 (sum(xf)/nel - 0.5).  Per step the inputs (x, g, dg) and the
    outputs (xnew, low, upp, gest, dk) are stored, for MMA2007 (8 steps), MMA1987 (5 steps) and the unconstrained
    form (objective only, 4 steps), so that the MMA update can be checked without the network, and for GCMMA
    (4 outer steps, whose inner iterations evaluate the network)."""
    out = {}
    for tag, version, constrained, steps in [("v2007", "MMA2007", True, 8), ("v1987", "MMA1987", True, 5),
                                             ("unc", "MMA2007", False, 4), ("gcmma", "GCMMA", True, 4)]:
        d = pym.VoxelDomain(30, 10)
        bc = np.concatenate([2 * d.nodes[0, :].flatten(), [2 * d.get_nodenumber(30, 0) + 1]])
        f = np.zeros(d.nnodes * 2)
        f[2 * d.get_nodenumber(0, 10) + 1] = -1.0
        sx = pym.Signal("x", np.full(d.nel, 0.5))
        with pym.Network() as fn:
            xf = pym.DensityFilter(d, radius=1.5)(sx)
            xs = pym.MathExpression("1e-9 + (1-1e-9)*inp0^3")(xf)
            K = pym.AssembleStiffness(d, bc=bc, plane="stress")(xs)
            u = pym.LinSolve(hermitian=True, symmetric=True)(K, f)
            c = pym.EinSum("i,i->")(u, f)
            g0 = pym.Scaling(scaling=100.0)(c)
            vol = pym.EinSum("i->")(xf)
            g1 = pym.MathExpression(f"10*(inp0/{d.nel} - 0.5)")(vol)
        resp = [g0, g1] if constrained else [g0]
        mma = pym.MMA(sx, resp, fn, move=0.2, verbosity=0, mmaversion=version)
        rec = {k: [] for k in ["x", "g", "dg", "xnew", "low", "upp", "offset", "gest", "dk"]}
        xval = mma.x
        for _ in range(steps):
            xnew, g, dg = mma.step(x=xval)
            for k, v in [("x", xval), ("g", g), ("dg", dg), ("xnew", xnew), ("low", mma.low), ("upp", mma.upp),
                         ("offset", mma.offset), ("gest", mma.gest), ("dk", mma.dk)]:
                rec[k].append(np.array(v, dtype=float).copy())
            xval = xnew
        for k, v in rec.items():
            out[f"{tag}_{k}"] = np.array(v)
        out[f"{tag}_bc"], out[f"{tag}_f"] = bc, f
    save("mma_mbb.npz", **out)


EINSUM_CASES = [("i,i->i", [(6,), (6,)]), ("i,j->ij", [(4,), (3,)]), ("ii->", [(5, 5)]), ("ij,j->i", [(4, 3), (3,)]),
                ("i,ij,j->", [(4,), (4, 3), (3,)]), ("ij,ij->ij", [(3, 4), (3, 4)]), ("ji,ij->ij", [(4, 3), (3, 4)]),
                ("ji,jk,kl->il", [(4, 2), (4, 3), (3, 2)]), ("ij->", [(3, 4)]), ("ijk,k->ij", [(2, 3, 4), (4,)])]


def einsums(pym):
    """pyMOTO's EinSum: responses and sensitivities (for a random output sensitivity) of the expressions in its
    docstring table and a few more."""
    out = {}
    rng = np.random.default_rng(23)
    for n, (expr, shapes) in enumerate(EINSUM_CASES):
        args = [rng.standard_normal(sh) for sh in shapes]
        m = pym.EinSum(expr)
        sig = [pym.Signal(f"a{i}", a) for i, a in enumerate(args)]
        y = m(*sig).state
        dy = rng.standard_normal(np.shape(y)) if np.ndim(y) else rng.standard_normal()
        ds = m._sensitivity(dy)
        ds = ds if isinstance(ds, list) else [ds]
        out[f"e{n}_y"], out[f"e{n}_dy"] = np.asarray(y), np.asarray(dy)
        for i, (a, d) in enumerate(zip(args, ds)):
            out[f"e{n}_a{i}"], out[f"e{n}_d{i}"] = a, np.asarray(d)
    save("einsum.npz", **out)


def filter_variants(pym):
    """FilterConv with constant-value (and mixed) boundary padding, and DensityFilter with `nonpadding`: outputs
    and adjoints of pyMOTO's own modules on random inputs."""
    out = {}
    cases = [("c3", (7, 5, 4), 2.5, dict(xmin_bc=0.0, xmax_bc=1.0, ymin_bc="edge", ymax_bc="wrap", zmin_bc=0.5,
                                         zmax_bc="symmetric")),
             ("c2", (9, 6), 2.0, dict(xmin_bc=1.0, xmax_bc="wrap", ymin_bc=0.0, ymax_bc=0.25)),
             ("c3b", (6, 6, 5), 1.5, dict(xmin_bc="wrap", xmax_bc="wrap", ymin_bc=0.0, ymax_bc=0.0, zmin_bc=1.0,
                                          zmax_bc=0.0))]
    for tag, shp, r, bcs in cases:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(11)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        fc = pym.FilterConv(d, radius=r, **bcs)
        sx = pym.Signal("x", x)
        sy = fc(sx)
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_r": np.array(r), f"{tag}_x": x, f"{tag}_dy": dy,
                    f"{tag}_y": sy.state, f"{tag}_dx": fc._sensitivity(dy)})
    # fixed values inside the domain (override_values), with and without a constant side
    for tag, shp, r, bcs, ovs in [("ov2", (9, 7), 2.0, {}, [((slice(0, 3), slice(2, 5), 0), 1.0),
                                                             ((np.array([6, 7]), np.array([1, 1]), 0), 0.0)]),
                                  ("ov3", (6, 5, 4), 1.5, dict(ymax_bc=0.3), [((slice(None), 0, slice(1, 3)), 0.7),
                                                                               ((2, slice(None), 3), 0.0)])]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(17)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        fc = pym.FilterConv(d, radius=r, **bcs)
        for idx, val in ovs:
            fc.override_values(idx, val)
        sy = fc(pym.Signal("x", x))
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_r": np.array(r), f"{tag}_x": x, f"{tag}_dy": dy,
                    f"{tag}_y": sy.state, f"{tag}_dx": fc._sensitivity(dy)})
    # fixed values in the padded array (override_padded_values): constant sides (the padding-filter example's
    # use), copies made by symmetric / edge / wrap padding, positions inside the domain, array values; later
    # calls win
    ring = [("po3", (8, 6, 5), 2.5, dict(xmin_bc=0, xmax_bc="symmetric", ymin_bc=0, ymax_bc=0, zmin_bc=0, zmax_bc=0),
             [(tuple(np.meshgrid(np.arange(2), 2 + np.arange(2, 4), 2 + np.arange(1, 4))), 1.0),
              ((slice(10, 12), slice(3, 6), slice(2, 5)), 0.3),
              ((np.array([3, 4]), np.array([4, 4]), np.array([3, 3])), 0.9),
              ((slice(0, 1), slice(4, 5), slice(3, 4)), 0.2)]),
            ("po2", (9, 7), 2.0, dict(xmin_bc="wrap", xmax_bc="wrap", ymin_bc="edge", ymax_bc=0.25),
             [((slice(0, 2), slice(0, 2), 0), 0.6),
              ((slice(None), 8, 0), 1.0),
              ((np.array([10, 5]), np.array([3, 0]), np.array([0, 0])), np.array([0.4, 0.7]))])]
    for tag, shp, r, bcs, povs in ring:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(19)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        fc = pym.FilterConv(d, radius=r, **bcs)
        for idx, val in povs:
            fc.override_padded_values(idx, val)
        sy = fc(pym.Signal("x", x))
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_r": np.array(r), f"{tag}_x": x, f"{tag}_dy": dy,
                    f"{tag}_y": sy.state, f"{tag}_dx": fc._sensitivity(dy), f"{tag}_xpad": fc.get_padded_vector(x)})
    for tag, shp, r in [("np2", (10, 6), 1.5), ("np3", (6, 5, 4), 2.0)]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(12)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        nonpad = np.sort(rng.choice(d.nel, d.nel // 3, replace=False))
        df = pym.DensityFilter(d, radius=r, nonpadding=nonpad)
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_r": np.array(r), f"{tag}_x": x, f"{tag}_dy": dy,
                    f"{tag}_nonpad": nonpad, f"{tag}_y": df(x), f"{tag}_dx": df._sensitivity(dy)})
    save("filter_variants.npz", **out)


def domain_helpers(pym):
    """VoxelDomain's geometry helpers: node / element indices and positions, connectivity, rigid body modes and
    shape functions (with derivatives) at seeded local points, for a 2D and a 3D domain with a moved origin."""
    out = {}
    rng = np.random.default_rng(13)
    for tag, shp, size, origin in [("d2", (5, 3, 0), (0.5, 0.25, 1.0), (1.0, -2.0, 0.0)),
                                   ("d3", (4, 3, 2), (0.1, 0.2, 0.3), (0.5, 0.0, -1.0))]:
        d = pym.VoxelDomain(*shp, *size)
        d.origin = np.array(origin)
        pts = (rng.uniform(-0.5, 0.5, (6, d.dim)) * np.array(size[:d.dim]))
        ii, jj, kk = rng.integers(0, shp[0], 5), rng.integers(0, shp[1], 5), rng.integers(0, max(shp[2], 1), 5)
        out.update({f"{tag}_pts": pts, f"{tag}_ijk": np.stack([ii, jj, kk]),
                    f"{tag}_node_idx": d.get_node_indices(), f"{tag}_node_pos": d.get_node_position(),
                    f"{tag}_el_idx": d.get_element_indices(), f"{tag}_el_pos": d.get_element_position(),
                    f"{tag}_econn": d.get_elemconnectivity(ii, jj, kk), f"{tag}_rbm": d.get_rigid_body_modes(),
                    f"{tag}_N": np.array([d.eval_shape_fun(p) for p in pts]),
                    f"{tag}_dN": np.array([d.eval_shape_fun_der(p) for p in pts]),
                    f"{tag}_domain_size": d.domain_size})
    save("domain_helpers.npz", **out)


def mass_matrices(pym):
    """AssembleMass element matrices (ndof 1 and dim, non-unit element sizes, density) and one assembled mass
    matrix with Dirichlet dofs applied to a seeded vector."""
    out = {}
    for tag, shp, size, ndof, rho in [("m2", (3, 2, 0), (0.5, 2.0, 0.3), 2, 7.8), ("m2s", (3, 2, 0), (1.0, 1.0, 1.0), 1, 1.0),
                                      ("m3", (2, 2, 2), (0.1, 0.2, 0.3), 3, 2.5), ("m3s", (2, 2, 2), (1.0, 0.5, 2.0), 1, 3.0)]:
        d = pym.VoxelDomain(*shp, *size)
        m = pym.AssembleMass(d, material_property=rho, ndof=ndof)
        out[f"{tag}_M0"] = m.el_mat
    d = pym.VoxelDomain(4, 3, 2, 0.5, 1.0, 1.5)
    rng = np.random.default_rng(14)
    x = rng.uniform(0.1, 1.0, d.nel)
    bc = np.array([0, 1, 2, 10, 44])
    sx = pym.Signal("x", x)
    M = pym.AssembleMass(d, bc=bc, material_property=2.0, ndof=3)(sx).state
    u = rng.standard_normal(M.shape[0])
    out.update({"asm_x": x, "asm_bc": bc, "asm_u": u, "asm_Mu": M @ u})
    save("mass.npz", **out)


def math_cases():
    """MathExpression cases: (name, expression, tags, inputs, output seed).  Pure numpy."""
    rng = np.random.default_rng(15)
    return [
        ("named", "sin(x)*y", ["x", "y"], [rng.uniform(0, 3, 3), 4.8], rng.standard_normal(3)),
        ("scalar", "10*(inp0/300 - 0.5)", ["vol"], [150.3], 1.0),
        ("vectors", "inp0^2 + inp1*inp0", ["a", "b"], [rng.standard_normal(4), rng.standard_normal(4)],
         rng.standard_normal(4)),
        ("bcast", "exp(-inp0)*inp1 + sqrt(inp1)", ["p", "q"], [rng.standard_normal((2, 3)),
                                                                      rng.uniform(0.1, 1, 3)],
         rng.standard_normal((2, 3))),
        ("simp", "1e-9 + (1-1e-9)*inp0^3", ["xf"], [0.37], 2.0),
        ("funcs", "tanh(inp0) + log(inp0 + 2)*cos(inp0) - atan(inp0)", [""], [rng.uniform(0, 1, 5)],
         rng.standard_normal(5)),
    ]


def math_expressions(pym):
    out = {}
    for name, expr, tags, inputs, seed in math_cases():
        sigs = [pym.Signal(t, v) for t, v in zip(tags, inputs)]
        m = pym.MathExpression(expr)
        so = m(*sigs)
        out[f"{name}_y"] = np.asarray(so.state)
        for i, d in enumerate(m._sensitivity(seed)):
            out[f"{name}_d{i}"] = np.asarray(d)
    save("math_expression.npz", **out)


def overhang_cases():
    """OverhangFilter cases: (name, shape, element size, direction, angle, nsampling).  Pure data."""
    return [("o2y", (12, 8, 0), (1.0, 1.0, 1.0), "y", 45.0, 8),
            ("o2x", (9, 10, 0), (1.0, 0.7, 1.0), "-x", 60.0, 8),
            ("o3z", (6, 5, 7), (1.0, 1.0, 1.0), "z", 45.0, 8),
            ("o3y", (5, 6, 4), (0.8, 1.0, 1.2), "-y", 50.0, 6)]


def overhang(pym):
    out = {}
    import contextlib
    import io
    for name, shp, size, direc, ang, ns in overhang_cases():
        d = pym.VoxelDomain(*shp, *size)
        rng = np.random.default_rng(16)
        x = rng.uniform(0.0, 1.0, d.nel)
        dy = rng.standard_normal(d.nel)
        with contextlib.redirect_stdout(io.StringIO()):   # the reference prints the support offsets
            m = pym.OverhangFilter(d, direction=direc, overhang_angle=ang, nsampling=ns)
            sx = pym.Signal("x", x)
            sy = m(sx)
            dx = m._sensitivity(dy)
        out.update({f"{name}_x": x, f"{name}_dy": dy, f"{name}_y": sy.state, f"{name}_dx": dx,
                    f"{name}_offsets": m.layer_offsets, f"{name}_origin": np.asarray(m.origin)})
    save("overhang.npz", **out)


def poisson(pym):
    """AssemblePoisson element matrices, and a thermal compliance network on a 6x4x4 grid (left face held at 0,
    uniform heat load, density-scaled conductivity): P u, the solution, the compliance and its sensitivities."""
    out = {}
    for tag, shp, size, k in [("p2", (3, 2, 0), (0.5, 2.0, 0.3), 2.5), ("p3", (2, 2, 2), (0.1, 0.2, 0.3), 1.7)]:
        out[f"{tag}_P0"] = pym.AssemblePoisson(pym.VoxelDomain(*shp, *size), material_property=k).poisson_element
    d = pym.VoxelDomain(6, 4, 4, 1.0, 0.5, 0.8)
    bc = d.nodes[0, :, :].flatten()
    f = np.full(d.nnodes, 1.0 / d.nnodes)
    rng = np.random.default_rng(18)
    x = rng.uniform(0.1, 1.0, d.nel)
    u_rand = rng.standard_normal(d.nnodes)
    sx = pym.Signal("x", x)
    with pym.Network() as fn:
        sK = pym.AssemblePoisson(d, bc=bc, material_property=2.0)(sx)
        su = pym.LinSolve(hermitian=True, symmetric=True)(sK, f)
        sc = pym.EinSum("i,i->")(su, f)
    fn.reset()
    sc.sensitivity = 1.0
    fn.sensitivity()
    out.update({"net_bc": bc, "net_f": f, "net_x": x, "net_Pu": sK.state @ u_rand, "net_urand": u_rand,
                "net_u": su.state, "net_c": np.array(float(sc.state)), "net_dx": sx.sensitivity.copy()})
    save("poisson.npz", **out)


def poisson_multigrid(pym):
    """GeometricMultigrid on one-component (AssemblePoisson) matrices, 3D and 2D: pyMOTO sizes the interpolation
    by the dofs per node of the matrix (one here).  Two levels with damped Jacobi (w = 0.6, 2 sweeps) over the
    automatically chosen direct coarsest solve: R, R^T P R and one V-cycle of a random residual."""
    out = {}
    for tag, shp in [("s3", (8, 4, 4)), ("s2", (8, 8))]:
        d = pym.VoxelDomain(*shp)
        rng = np.random.default_rng(19)
        x = rng.uniform(1e-3, 1.0, d.nel)
        bc = d.nodes[0, ...].flatten()
        P = pym.AssemblePoisson(d, bc=bc)(x)
        mg1 = pym.solvers.GeometricMultigrid(d, smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2)
        mg2 = pym.solvers.GeometricMultigrid(mg1.sub_domain, smoother=pym.solvers.DampedJacobi(w=0.6), smooth_steps=2)
        mg1.inner_level = mg2
        mg1.update(P)
        R = mg1.R.tocoo()
        Ac = mg2.A.tocsr()
        Ac.eliminate_zeros()
        r = rng.standard_normal(P.shape[0])
        r[bc] = 0.0
        z = mg1.solve(r)
        out.update({f"{tag}_shape": np.array(shp), f"{tag}_x": x, f"{tag}_bc": bc,
                    f"{tag}_R_row": R.row, f"{tag}_R_col": R.col, f"{tag}_R_val": R.data,
                    f"{tag}_Ac_data": Ac.data, f"{tag}_Ac_indices": Ac.indices, f"{tag}_Ac_indptr": Ac.indptr,
                    f"{tag}_r": r, f"{tag}_z": z})
    save("poisson_mg.npz", **out)


def springs(pym):
    """Springs to ground through AssembleStiffness(add_constant=...) (pymoto/modules/assembly.py:294-295, the
    compliant-mechanism example's use): 2D (mechanism-like supports, springs at an input and an output dof) and
    3D (cantilever with springs on the loaded face, one on a Dirichlet dof); K u, the solution, compliance and
    its sensitivities.  A 3D case without any Dirichlet dof (soft supports only, as the self-weight example)."""
    import scipy.sparse as sps
    out = {}
    cases = [("q4", (12, 6), (12, 6, 0)), ("h8", (8, 4, 4), (8, 4, 4)), ("soft", (6, 4, 4), (6, 4, 4))]
    for tag, shp, shp3 in cases:
        d = pym.VoxelDomain(*shp)
        dim = 2 if len(shp) == 2 else 3
        rng = np.random.default_rng({"q4": 31, "h8": 32, "soft": 33}[tag])
        x = rng.uniform(0.1, 1.0, d.nel)
        f = np.zeros(d.nnodes * dim)
        if tag == "q4":
            left = d.get_nodenumber(0, np.arange(shp[1] + 1))
            right = d.get_nodenumber(shp[0], np.arange(shp[1] + 1))
            bc = np.union1d(left * 2, (right[:, None] * 2 + np.arange(2)).ravel())
            din, dout = 2 * left[0] + 1, 2 * left[-1] + 1
            f[din] = 1.0
            idx, val = np.array([din, dout]), np.array([10.0, 10.0])
        elif tag == "h8":
            left = d.nodes[0, :, :].flatten()
            bc = (left[:, None] * 3 + np.arange(3)).ravel()
            tip = d.get_nodenumber(shp[0], shp[1] // 2, shp[2] // 2)
            f[3 * tip + 1] = -1.0
            idx = np.array([3 * tip + 1, 3 * tip, bc[4]])
            val = np.array([0.5, 2.0, 3.0])
        else:
            bc = None
            corners = [d.get_nodenumber(0, j, k) for j in (0, shp[1]) for k in (0, shp[2])]
            idx = np.array([3 * n + c for n in corners for c in range(3)])
            val = np.full(idx.size, 5.0)
            f[3 * d.get_nodenumber(shp[0], shp[1] // 2, shp[2] // 2) + 1] = -1.0
        K_const = sps.csc_matrix((val, (idx, idx)), shape=(d.nnodes * dim, d.nnodes * dim))
        sx = pym.Signal("x", x)
        with pym.Network() as fn:
            sK = pym.AssembleStiffness(d, bc=bc, add_constant=K_const)(sx)
            su = pym.LinSolve(hermitian=True, symmetric=True)(sK, f)
            sc = pym.EinSum("i,i->")(su, f)
        fn.reset()
        sc.sensitivity = 1.0
        fn.sensitivity()
        u_rand = rng.standard_normal(d.nnodes * dim)
        out.update({f"{tag}_shape": np.array(shp3), f"{tag}_bc": np.zeros(0, np.int64) if bc is None else bc,
                    f"{tag}_x": x, f"{tag}_f": f, f"{tag}_idx": idx, f"{tag}_val": val,
                    f"{tag}_urand": u_rand, f"{tag}_Ku": sK.state @ u_rand, f"{tag}_u": su.state,
                    f"{tag}_c": np.array(float(sc.state)), f"{tag}_dx": sx.sensitivity.copy()})
    save("springs.npz", **out)


def vti_cases():
    """The VTI output cases: (name, (nelx, nely, nelz), element size, origin, scale, vectors).  Pure numpy, so
    the tests rebuild the same inputs without pyMOTO."""
    rng = np.random.default_rng(20251204)
    cases = []
    nel, nn = 4 * 3 * 2, 5 * 4 * 3
    cases.append(("h8", (4, 3, 2), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), 1.0, {
        "u": rng.standard_normal(3 * nn),
        "x": rng.random(nel),
        "modes": rng.standard_normal((11, 3 * nn)),         # point block vector, two-digit suffixes
        "fields": rng.random((nel, 2)),                     # cell block vector along the second axis
        "z": rng.standard_normal(nn) + 1j * rng.standard_normal(nn),
        "bad": rng.random(7),                               # neither cell nor point data: skipped
    }))
    nel, nn = 5 * 3, 6 * 4
    cases.append(("q4", (5, 3, 0), (0.5, 0.25, 1.0), (1.0, -2.0, 0.0), 2.5, {
        "u": rng.standard_normal(2 * nn),                   # padded to three components
        "uc": rng.standard_normal(2 * nn) + 1j * rng.standard_normal(2 * nn),
        "x": rng.random(nel).astype(np.float32),
        "xc": rng.random((3, nel)) + 1j * rng.random((3, nel)),
    }))
    return cases


def scalar_cases():
    """ScalarToFile cases: (name, saveto, fmt, separator, states per iteration {tag: value}).  Pure numpy."""
    rng = np.random.default_rng(20251205)
    it = []
    for k in range(3):
        it.append({"compliance": float(rng.uniform(1, 100)), "volume": np.float64(rng.uniform(0, 1)),
                   "eig": rng.standard_normal(3), "block": rng.standard_normal((2, 2)), "count": 7 + k})
    return [("txt", "scalars_txt.txt", ".10e", "\t", it), ("csv", "scalars_csv.csv", ".3f", "\t", it)]


def scalar_files(pym):
    for name, fname, fmt, sep, its in scalar_cases():
        sigs = [pym.Signal(tag, val) for tag, val in its[0].items()]
        with pym.Network() as fn:
            pym.ScalarToFile(os.path.join(OUT, fname), fmt=fmt, separator=sep)(*sigs)
        for vals in its[1:]:
            for sg in sigs:
                sg.state = vals[sg.tag]
            fn.response()
        print("wrote", fname)


def vti_files(pym):
    for name, shp, size, origin, scale, vecs in vti_cases():
        d = pym.VoxelDomain(*shp, *size)
        d.origin = np.array(origin)
        d.write_to_vti(vecs, filename=os.path.join(OUT, f"vti_{name}.vti"), scale=scale)
        print("wrote", f"vti_{name}.vti")


if __name__ == "__main__":
    warnings.filterwarnings("ignore")
    argv = sys.argv[1:]
    if "--reference" in argv:
        i = argv.index("--reference")
        REF = argv[i + 1]
        del argv[i:i + 2]
    pym = import_reference()
    which = argv or ["all"]
    if "all" in which:
        maps_and_k0(pym)
        assembly(pym)
        filters(pym)
        multigrid(pym)
        pipeline(pym, "h8_mg", (8, 4, 4), "conv", 1.5, 3, 1e-8)
        pipeline(pym, "q4_mg", (16, 8), "density", 2.0, 3, 1e-8, plane="stress")
        pipeline(pym, "h8_direct", (6, 4, 2), "density", 1.5, 0, 1e-8)
        oc_mbb(pym)
    if "all" in which or "springs" in which:
        springs(pym)
    if "all" in which or "vti" in which:
        vti_files(pym)
    if "all" in which or "mma" in which:
        mma_mbb(pym)
    if "all" in which or "scalars" in which:
        scalar_files(pym)
    if "all" in which or "filters2" in which:
        filter_variants(pym)
    if "all" in which or "domain" in which:
        domain_helpers(pym)
    if "all" in which or "mass" in which:
        mass_matrices(pym)
    if "all" in which or "math" in which:
        math_expressions(pym)
    if "all" in which or "overhang" in which:
        overhang(pym)
    if "all" in which or "poisson" in which:
        poisson(pym)
    if "all" in which or "poisson_mg" in which:
        poisson_multigrid(pym)
    if "all" in which or "einsum" in which:
        einsums(pym)
