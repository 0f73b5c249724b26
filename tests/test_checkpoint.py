"""Checkpoint and resume: the .npz round trip of nested states (CPU), and on the GPU a resumed FP64 design run
that reproduces the uninterrupted run bit for bit."""
import numpy as np
import pytest
import torch

import pymoto_gb300 as pg
from pymoto_gb300.checkpoint import load_checkpoint, save_checkpoint


class _Holder:
    def __init__(self, sd=None):
        self.sd = sd

    def state_dict(self):
        return self.sd

    def load_state_dict(self, sd):
        self.sd = sd


def test_nested_states_round_trip_bit_for_bit(tmp_path):
    rng = np.random.default_rng(0)
    sd = {"a": torch.randn(5, dtype=torch.float64), "b": torch.randn(7).to(torch.bfloat16),
          "c": np.arange(6).reshape(2, 3), "d": [torch.ones(2), torch.zeros(3)], "e": None, "f": 3,
          "g": [1.5, 2.5], "h": {"x": torch.tensor([1, 2, 3]), "y": "name"}, "rng": rng.bit_generator.state}
    save_checkpoint(tmp_path / "c.npz", obj=_Holder(sd))
    h = _Holder()
    load_checkpoint(tmp_path / "c.npz", device=None, obj=h)
    r = h.sd
    assert torch.equal(r["a"], sd["a"]) and r["a"].dtype == torch.float64
    assert r["b"].dtype == torch.bfloat16 and torch.equal(r["b"].view(torch.int16), sd["b"].view(torch.int16))
    np.testing.assert_array_equal(r["c"], sd["c"])
    assert torch.equal(r["d"][0], sd["d"][0]) and torch.equal(r["d"][1], sd["d"][1])
    assert r["e"] is None and r["f"] == 3 and r["g"] == [1.5, 2.5]
    assert torch.equal(r["h"]["x"], sd["h"]["x"]) and r["h"]["y"] == "name"
    g2 = np.random.default_rng(99)
    g2.bit_generator.state = r["rng"]
    assert g2.random() == rng.random()


def test_optimizer_solver_and_signal_states(tmp_path):
    from pymoto_gb300.core import Network, Signal
    sx = Signal("x", np.linspace(0.1, 0.9, 6))
    oc = pg.OC(sx, Signal("c", 1.0), Network(), verbosity=0)
    oc.iter, oc.history, oc.maxvol = 7, [3.0, 2.5, 2.25], 0.4
    ls = pg.LinSolve()
    ls.u = np.arange(4.0)
    save_checkpoint(tmp_path / "s.npz", x=sx, oc=oc, solve=ls)
    sx2, oc2, ls2 = Signal("x", None), pg.OC(Signal("x", np.zeros(6)), Signal("c"), Network()), pg.LinSolve()
    load_checkpoint(tmp_path / "s.npz", device=None, x=sx2, oc=oc2, solve=ls2)
    np.testing.assert_array_equal(sx2.state, sx.state)
    assert (oc2.iter, oc2.history, oc2.maxvol) == (7, [3.0, 2.5, 2.25], 0.4)
    np.testing.assert_array_equal(ls2.u, ls.u)


@pytest.mark.gpu
def test_resumed_fp64_run_reproduces_the_uninterrupted_run(tmp_path):
    import oracle as O
    from conftest import clamp_face_dofs
    from test_gpu_pipeline import build_network
    shape = (16, 8, 8)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0

    def run():
        _, sx, _, sc, fn = build_network(pg, shape, bc, f, "conv", 1.5, 3, 1e-10, state_kind="torch")
        ls = next(m for m in fn if isinstance(m, pg.LinSolve))
        return sx, sc, fn, ls, pg.OC(sx, sc, fn, move=0.2, verbosity=0)

    sx, sc, fn, ls, oc = run()
    for _ in range(3):
        oc.step()
    save_checkpoint(tmp_path / "run.npz", x=sx, oc=oc, solve=ls)
    for _ in range(2):
        oc.step()
    ref = oc.history[-2:]
    sx2, sc2, fn2, ls2, oc2 = run()
    load_checkpoint(tmp_path / "run.npz", x=sx2, oc=oc2, solve=ls2)
    for _ in range(2):
        oc2.step()
    assert oc2.history[-2:] == ref          # bit for bit


@pytest.mark.gpu
def test_learned_warm_start_state_round_trip(tmp_path):
    from pymoto_gb300.learned import LearnedWarmStart
    a = LearnedWarmStart((32, 16, 16), seed=1)      # stride 4: voxel grid (8, 4, 4)
    b = LearnedWarmStart((32, 16, 16), seed=2)
    a.rng.random()
    save_checkpoint(tmp_path / "l.npz", ws=a)
    load_checkpoint(tmp_path / "l.npz", ws=b)
    assert torch.equal(a.net.w, b.net.w) and torch.equal(a.net.w_bf, b.net.w_bf)
    assert a.rng.random() == b.rng.random()


@pytest.mark.gpu
def test_resumed_mma_run_reproduces_the_uninterrupted_run(tmp_path, golden):
    """MMA keeps asymptote offsets and the two previous designs; a resumed run continues bit for bit."""
    g = golden("mma_mbb.npz")

    def build():
        d = pg.VoxelDomain(30, 10)
        f = torch.from_numpy(g["v2007_f"]).cuda()
        sx = pg.Signal("x", torch.full((d.nel,), 0.5, dtype=torch.float64, device="cuda"))
        with pg.Network() as fn:
            xf = pg.DensityFilter(d, radius=1.5)(sx)
            xs = pg.SIMP(xmin=1e-9, penal=3.0)(xf)
            K = pg.AssembleStiffness(d, bc=g["v2007_bc"], plane="stress")(xs)
            ls = pg.LinSolve(hermitian=True, symmetric=True)
            u = ls(K, f)
            c = pg.EinSum("i,i->")(u, f)
            s0 = pg.Scaling(scaling=100.0)
            g0 = s0(c)
            g1 = pg.Scaling(scaling=5.0, maxval=0.5 * d.nel)(pg.EinSum("i->")(xf))
        return sx, ls, s0, pg.MMA(sx, [g0, g1], fn, move=0.2, verbosity=0)

    sx, ls, s0, mma = build()
    xval = mma.x
    for _ in range(3):
        xval, _, _ = mma.step(x=xval)
    mma.x = xval
    save_checkpoint(tmp_path / "mma.npz", x=sx, mma=mma, solve=ls, scale=s0)
    ref = []
    for _ in range(2):
        xval, gk, _ = mma.step(x=xval)
        ref.append(gk.cpu().numpy())
    sx2, ls2, s02, mma2 = build()
    load_checkpoint(tmp_path / "mma.npz", x=sx2, mma=mma2, solve=ls2, scale=s02)
    xval = mma2.x
    for k in range(2):
        xval, gk, _ = mma2.step(x=xval)
        np.testing.assert_array_equal(gk.cpu().numpy(), ref[k])
