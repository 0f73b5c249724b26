"""Learned warm start: network kernels against a torch-CPU FP64 reference of the same architecture (with the
BF16 storage of weights and activations emulated), and the warm start inside the FP64 flexible CG."""
import numpy as np
import pytest
import torch
import torch.nn.functional as Fn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import pymoto_gb300 as pg
    from pymoto_gb300 import _lib
    _lib.load()
    return pg


def bf(t):
    return t.to(torch.bfloat16).to(torch.float64)


def _weights(net, name):
    """(cout, cin, 3, 3, 3) FP64 weights (BF16-rounded) and bias of one layer, from w[tap][cin][cout]."""
    o, cin, cout = net.offsets[name]
    w = net.w.detach().cpu().double()
    W = bf(w[o:o + 27 * cin * cout]).reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous()
    b = w[o + 27 * cin * cout:o + 27 * cin * cout + cout].clone()
    return W, b


def _to_cdhw(flat, grid, c):
    nx, ny, nz = grid
    return flat.reshape(nz, ny, nx, c).permute(3, 0, 1, 2)


def _vox_to_node(vox):
    """(3, nz, ny, nx) voxel values -> (3, nz+1, ny+1, nx+1) nodal averages of the adjacent voxels."""
    c, nz, ny, nx = vox.shape
    pad = Fn.pad(vox, (1, 1, 1, 1, 1, 1))
    ones = Fn.pad(torch.ones((1, nz, ny, nx), dtype=vox.dtype), (1, 1, 1, 1, 1, 1))
    k = torch.ones((1, 1, 2, 2, 2), dtype=vox.dtype)
    s = Fn.conv3d(pad.reshape(c, 1, nz + 2, ny + 2, nx + 2), k).reshape(c, nz + 1, ny + 1, nx + 1)
    cnt = Fn.conv3d(ones.reshape(1, 1, nz + 2, ny + 2, nx + 2), k).reshape(1, nz + 1, ny + 1, nx + 1)
    return s / cnt


def torch_forward(net, feat):
    """The network in FP64 autograd, BF16 rounding where the device stores BF16."""
    g1 = net.g1
    params = {}
    for name in ["enc1a", "enc1b", "enc2a", "enc2b", "enc3a", "enc3b", "dec2", "dec1", "head"]:
        W, b = _weights(net, name)
        params[name] = (W.requires_grad_(True), b.requires_grad_(True))

    def conv(name, x, relu=True):
        W, b = params[name]
        y = Fn.conv3d(x.unsqueeze(0), W, b, padding=1).squeeze(0)
        if relu:
            y = torch.relu(y)
            y = y + (bf(y.detach()) - y.detach())          # stored as BF16 (straight-through rounding)
        return y

    def up(x):
        return x.repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3)

    def pool(x):
        p = Fn.avg_pool3d(x.unsqueeze(0), 2).squeeze(0)
        return p + (bf(p.detach()) - p.detach())

    x = _to_cdhw(bf(feat.detach().cpu().float().double()), g1, 4)
    a1 = conv("enc1a", x)
    a2 = conv("enc1b", a1)
    a3 = conv("enc2a", pool(a2))
    a4 = conv("enc2b", a3)
    a5 = conv("enc3a", pool(a4))
    a6 = conv("enc3b", a5)
    a7 = conv("dec2", torch.cat([a4, up(a6)], 0))
    a8 = conv("dec1", torch.cat([a2, up(a7)], 0))
    out = conv("head", a8, relu=False)
    return out, params


def _flat_grad(net, params):
    g = torch.zeros(net.nparam, dtype=torch.float64)
    for name, (W, b) in params.items():
        o, cin, cout = net.offsets[name]
        g[o:o + 27 * cin * cout] = W.grad.permute(2, 3, 4, 1, 0).reshape(-1)
        g[o + 27 * cin * cout:o + 27 * cin * cout + cout] = b.grad
    return g


def test_network_forward_backward_matches_torch(pg):
    from pymoto_gb300._lib import call, stream
    from pymoto_gb300.learned import ConvNet3D
    grid = (8, 4, 4)
    net = ConvNet3D(grid, seed=3)
    rng = np.random.default_rng(0)
    feat = torch.from_numpy(rng.uniform(-1, 1, net.v1 * 4)).to("cuda", torch.bfloat16)
    net.feat.copy_(feat)
    out = net.forward()
    ref, params = torch_forward(net, feat)
    out_t = _to_cdhw(out.detach().cpu().double(), grid, 3)
    assert torch.linalg.norm(out_t - ref.detach()) <= 1e-2 * torch.linalg.norm(ref.detach())
    # loss on the nodes: sum (V2N(out) - target)^2
    nodes_ref = _vox_to_node(ref)
    target = torch.from_numpy(rng.standard_normal(nodes_ref.numel())).double()
    tgt_nodes = target.reshape(nodes_ref.shape[1], nodes_ref.shape[2], nodes_ref.shape[3], 3).permute(3, 0, 1, 2)
    loss_ref = ((nodes_ref - tgt_nodes) ** 2).sum()
    loss_ref.backward()
    pred = torch.empty(nodes_ref.numel(), dtype=torch.float64, device="cuda")
    call("pmg_nn_vox_to_node", 0, *grid, net.out, pred, stream())
    np.testing.assert_allclose(pred.cpu().numpy().reshape(-1, 3).T.reshape(nodes_ref.shape),
                               _vox_to_node(out_t).numpy(), rtol=1e-6, atol=1e-7)
    dpred = torch.empty(nodes_ref.numel(), dtype=torch.float32, device="cuda")
    parts = torch.zeros((pred.numel() + 255) // 256, dtype=torch.float64, device="cuda")
    call("pmg_nn_mse", pred.numel(), pred, target.cuda(), 1.0, dpred, parts, stream())
    assert abs(parts.sum().item() - loss_ref.item()) <= 2e-2 * loss_ref.item()
    call("pmg_nn_vox_to_node", 1, *grid, dpred, net.d_out, stream())
    g = net.backward().detach().cpu().double()
    gr = _flat_grad(net, params)
    for name in params:
        o, cin, cout = net.offsets[name]
        sl = slice(o, o + 27 * cin * cout + cout)
        a, b = g[sl], gr[sl]
        rel = torch.linalg.norm(a - b) / torch.linalg.norm(b)
        cos = torch.dot(a, b) / (torch.linalg.norm(a) * torch.linalg.norm(b))
        assert rel <= 5e-2 and cos >= 0.999, (name, float(rel), float(cos))


def test_layout_kernels_exact(pg):
    """pool / upsample / concat / voxel-to-node / injection against numpy, exactly (dyadic values)."""
    from pymoto_gb300._lib import call, stream
    rng = np.random.default_rng(1)
    cg, c = (2, 3, 2), 5
    fg = tuple(2 * v for v in cg)
    nvf, nvc = int(np.prod(fg)), int(np.prod(cg))
    xf = rng.integers(-8, 8, nvf * c).astype(np.float32)
    t = torch.from_numpy(xf).to("cuda", torch.bfloat16)
    out = torch.empty(nvc * c, dtype=torch.bfloat16, device="cuda")
    call("pmg_nn_pool2", 0, *cg, c, t, out, stream())
    X = xf.reshape(fg[2], fg[1], fg[0], c)
    P = X.reshape(cg[2], 2, cg[1], 2, cg[0], 2, c).mean(axis=(1, 3, 5))
    np.testing.assert_array_equal(out.float().cpu().numpy(), P.reshape(-1))
    d = torch.from_numpy(rng.integers(-8, 8, nvc * c).astype(np.float32)).cuda()
    din = torch.ones(nvf * c, dtype=torch.float32, device="cuda")
    call("pmg_nn_pool2", 1, *cg, c, d, din, stream())       # adds 1/8 of the coarse gradient
    D = d.cpu().numpy().reshape(cg[2], cg[1], cg[0], c)
    ref = 1.0 + np.repeat(np.repeat(np.repeat(D, 2, 0), 2, 1), 2, 2) / 8
    np.testing.assert_array_equal(din.cpu().numpy(), ref.reshape(-1))
    # upsample into channels [2, 2+c) of a (c+2)-channel tensor, and its adjoint
    cat = torch.zeros(nvf * (c + 2), dtype=torch.bfloat16, device="cuda")
    call("pmg_nn_up2", 0, *cg, c, c + 2, 2, d.to(torch.bfloat16), cat, stream())
    C = cat.float().cpu().numpy().reshape(fg[2], fg[1], fg[0], c + 2)
    np.testing.assert_array_equal(C[..., 2:], np.repeat(np.repeat(np.repeat(D, 2, 0), 2, 1), 2, 2))
    dc = torch.from_numpy(rng.integers(-8, 8, nvf * (c + 2)).astype(np.float32)).cuda()
    dcoarse = torch.empty(nvc * c, dtype=torch.float32, device="cuda")
    call("pmg_nn_up2", 1, *cg, c, c + 2, 2, dc, dcoarse, stream())
    DC = dc.cpu().numpy().reshape(fg[2], fg[1], fg[0], c + 2)[..., 2:]
    np.testing.assert_array_equal(dcoarse.cpu().numpy(),
                                  DC.reshape(cg[2], 2, cg[1], 2, cg[0], 2, c).sum(axis=(1, 3, 5)).reshape(-1))
    # concat copy and split
    cat2 = torch.zeros(nvc * (c + 3), dtype=torch.bfloat16, device="cuda")
    call("pmg_nn_copy_channels", nvc, c, c + 3, 1, d.to(torch.bfloat16), cat2, stream())
    np.testing.assert_array_equal(cat2.float().cpu().numpy().reshape(nvc, c + 3)[:, 1:1 + c], d.cpu().numpy().reshape(nvc, c))
    dsk = torch.ones(nvc * c, dtype=torch.float32, device="cuda")
    g2 = torch.from_numpy(rng.integers(-8, 8, nvc * (c + 3)).astype(np.float32)).cuda()
    call("pmg_nn_split_channels", nvc, c, c + 3, 1, g2, dsk, stream())
    np.testing.assert_array_equal(dsk.cpu().numpy().reshape(nvc, c), 1 + g2.cpu().numpy().reshape(nvc, c + 3)[:, 1:1 + c])
    # injection of a fine nodal field at stride 2
    nx, ny, nz = 4, 2, 2
    uf = torch.from_numpy(rng.standard_normal((nx + 1) * (ny + 1) * (nz + 1) * 3)).cuda()
    uc = torch.empty((nx // 2 + 1) * (ny // 2 + 1) * (nz // 2 + 1) * 3, dtype=torch.float64, device="cuda")
    call("pmg_nn_inject", nx, ny, nz, 2, uf, 2.0, uc, stream())
    U = uf.cpu().numpy().reshape(nz + 1, ny + 1, nx + 1, 3)
    np.testing.assert_array_equal(uc.cpu().numpy(), 2.0 * U[::2, ::2, ::2].reshape(-1))


def test_adam_matches_reference(pg):
    from pymoto_gb300._lib import call, stream
    rng = np.random.default_rng(2)
    n = 1000
    w = rng.standard_normal(n).astype(np.float32)
    m = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    wd = torch.from_numpy(w).cuda()
    md, vd = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    wb = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    lr, b1, b2, eps = 1e-2, 0.9, 0.999, 1e-8
    for step in range(1, 4):
        g = rng.standard_normal(n).astype(np.float32)
        call("pmg_nn_adam", n, wd, torch.from_numpy(g).cuda(), md, vd, wb, lr, b1, b2, eps, step, 0.0, stream())
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        w = w - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    np.testing.assert_allclose(wd.cpu().numpy(), w, rtol=1e-5, atol=1e-6)
    assert torch.equal(wb.cpu(), wd.to(torch.bfloat16).cpu())


def test_training_reduces_the_loss(pg):
    """A few Adam steps on one (field, solution) pair reduce the training loss."""
    from pymoto_gb300.learned import LearnedWarmStart
    ws = LearnedWarmStart((16, 8, 8), stride=2, capacity=1, train_steps=0, lr=3e-3, seed=0)
    rng = np.random.default_rng(4)
    A = _operator(pg, (16, 8, 8), rng)
    kk, jj, ii = np.meshgrid(np.arange(9), np.arange(9), np.arange(17), indexing="ij")
    u = np.stack([np.sin(0.2 * ii) * jj, 0.1 * ii ** 2 / 16, np.cos(0.3 * kk) * ii], -1).reshape(-1)
    ws.observe(A, torch.from_numpy(u).cuda())
    ws.train_step(0)
    l0 = ws.loss()
    for _ in range(60):
        ws.train_step(0)
    assert ws.loss() < 0.3 * l0


def _operator(pg, shape, rng):
    from conftest import clamp_face_dofs
    import oracle as O
    from pymoto_gb300.operators import bc_node_mask
    g = O.Grid(*shape)
    x = 1e-9 + (1 - 1e-9) * rng.uniform(0.2, 1.0, g.nel) ** 3
    K0 = O.element_stiffness(g)
    bcd = clamp_face_dofs(g)
    mask = torch.from_numpy(bc_node_mask(g.nnodes, g.dim, bcd)).to("cuda", torch.uint8)
    return pg.StiffnessOperator(pg.Grid(*shape), torch.from_numpy(x).cuda(), K0, mask, O.default_bcdiagval(K0))


def test_learned_warm_start_gain(pg):
    """What the trained network gains: FCG iterations over a sequence of designs of an OC run, with the
    learned warm start (Rayleigh-Ritz with the previous solution) and without it (previous solution
    only).  Both reach the same FP64 relative residual; the learned run may not take more iterations."""
    import oracle as O
    from conftest import clamp_face_dofs
    from pymoto_gb300.learned import LearnedWarmStart
    shape = (32, 16, 16)
    d = pg.VoxelDomain(*shape)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    nnx, nny = shape[0] + 1, shape[1] + 1
    f[3 * (((shape[2] // 2) * nny + shape[1] // 2) * nnx + shape[0]) + 1] = -1.0
    results = {}
    active = []
    for learned in (False, True, "cc"):
        rng = np.random.default_rng(7)
        sx = pg.Signal("x", torch.from_numpy(rng.uniform(0.2, 0.8, g.nel)).cuda())
        mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smooth_steps=2, coarse_smooth_steps=3, precision="fp32",
                                              smoother="chebyshev")
        ws = LearnedWarmStart(shape, stride=4, capacity=8, train_steps=4, lr=2e-3,
                              coarse_correction=learned == "cc") if learned else None
        solver = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-6, m=1, warm_start=ws)
        with pg.Network() as fn:
            xf = pg.FilterConv(d, radius=2.0)(sx)
            xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
            K = pg.AssembleStiffness(d, bc=bc)(xs)
            u = pg.LinSolve(hermitian=True, symmetric=True, solver=solver)(K, torch.from_numpy(f).cuda())
            c = pg.EinSum("i,i->")(u, torch.from_numpy(f).cuda())
        oc = pg.OC(sx, c, fn, move=0.2, verbosity=0)
        its = []
        for _ in range(12):
            oc.step()
            its.append(solver.iterations)
            assert solver.last_residual <= 1e-6
            if learned == "cc":
                active.append(float(solver._fcg["learned_cc"][4]) > 0.0)
        results[learned] = its
    base, lrn, lcc = results[False], results[True], results["cc"]
    print(f"FCG iterations per design without / with the learned warm start / with it and the learned coarse "
          f"correction: {base} / {lrn} / {lcc}")
    # the network starts untrained: compare the designs after the first few
    assert sum(lrn[4:]) <= sum(base[4:])
    # the one-dimensional learned coarse space (deflation) was in use and the solves still reach the FP64
    # tolerance without more than a few extra iterations
    assert any(active) and sum(lcc[4:]) <= sum(base[4:]) + 4


def test_pretrained_network_on_cold_solves(pg):
    """What the trained network gains where the solver has no previous solution to start from (the first
    design of a run): trained on the solutions of 48 seeded smoothed-noise density fields, its prediction w of 6
    unseen fields is scored by the share of the solution's energy it captures, (b.w)^2 / (w.Kw b.u*) (the
    Rayleigh-Ritz multiple of w then has the energy error sqrt(1 - share) of the zero start), and it starts the
    FP64 flexible CG.  Measured on GB300: the prediction carries 3-5 % of the energy and the solves take the
    same iterations as from zero.  Under a point load most of the solution's energy sits in the load's local
    response (the compliance is the load-point displacement), which a prediction on the coarse voxels cannot
    represent and the multigrid removes within its first iterations from either start.  The test pins that
    the network learned the global response (a share above 1 % for every unseen field) and that starting from
    it never costs iterations; the times are printed."""
    from scipy.ndimage import gaussian_filter
    import oracle as O
    from conftest import clamp_face_dofs
    from pymoto_gb300.learned import LearnedWarmStart
    from pymoto_gb300.operators import bc_node_mask
    shape = (32, 16, 16)
    g = O.Grid(*shape)
    d = pg.VoxelDomain(*shape)
    K0 = O.element_stiffness(g)
    mask = torch.from_numpy(bc_node_mask(g.nnodes, g.dim, clamp_face_dofs(g))).to("cuda", torch.uint8)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(shape[0], shape[1] // 2, shape[2] // 2) + 1] = -1.0
    b = torch.from_numpy(f).cuda()

    def operator(seed):
        a = gaussian_filter(np.random.default_rng(seed).uniform(0.0, 1.0, shape[::-1]), sigma=2.0)
        a = 1e-3 + (1.0 - 1e-3) * (a - a.min()) / (a.max() - a.min())
        x = 1e-9 + (1 - 1e-9) * a.ravel() ** 3
        return pg.StiffnessOperator(pg.Grid(*shape), torch.from_numpy(x).cuda(), K0, mask,
                                    O.default_bcdiagval(K0))

    ws = LearnedWarmStart(shape, stride=2, capacity=48, train_steps=6, lr=2e-3, history=0, seed=0)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=3, smooth_steps=2, coarse_smooth_steps=3, precision="fp32",
                                          smoother="chebyshev")
    trainer = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-8, m=1)
    for seed in range(48):
        A = operator(1000 + seed)
        trainer.update(A)
        ws.observe(A, trainer.solve(b))
    for _ in range(200):                             # a few passes over the stored pairs
        ws.train_step(int(ws.rng.integers(48)))
    ws.sync_training()
    print(f"training loss (squared error of a unit-norm target) after pretraining: {ws.loss():.3e}")
    ws.train_steps = 0                               # evaluation: the test fields' solutions are not learned

    shares, its, times = [], {False: [], True: []}, {False: 0.0, True: 0.0}
    for seed in range(6):
        A = operator(5000 + seed)
        exact = pg.MixedPrecisionCG(preconditioner=mgs[0], tol=1e-10, m=1)
        exact.update(A)
        ustar = exact.solve(b)
        w = torch.empty_like(b)
        pg._lib.call("pmg_mask_bc", pg._lib.F64, 3, g.nnodes, mask, 0, ws.predict(A), w, pg._lib.stream())
        share = float(torch.dot(b, w)) ** 2 / (float(torch.dot(w, A.matvec(w))) * float(torch.dot(b, ustar)))
        shares.append(share)
        for learned in (False, True):
            mg = pg.GeometricMultigrid.hierarchy(d, levels=3, smooth_steps=2, coarse_smooth_steps=3,
                                                 precision="fp32", smoother="chebyshev")
            solver = pg.MixedPrecisionCG(preconditioner=mg[0], tol=1e-6, m=1, warm_start=ws if learned else None)
            solver.update(A)
            solver.solve(b)                          # warm-up (graph capture, kernel loading)
            solver.update(A)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            solver.solve(b)
            e1.record()
            torch.cuda.synchronize()
            assert solver.last_residual <= 1e-6
            its[learned].append(solver.iterations)
            times[learned] += e0.elapsed_time(e1)
    print(f"cold solves: energy share of the prediction {np.round(shares, 3)}; FCG iterations without / with the "
          f"pretrained network: {its[False]} / {its[True]}; time {times[False]:.2f} / {times[True]:.2f} ms")
    assert min(shares) > 0.01
    assert sum(its[True]) <= sum(its[False])
