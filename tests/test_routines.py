"""finite_difference and the network cone helpers of the standalone runtime (CPU, numpy modules)."""
import numpy as np
import pytest

import pymoto_gb300 as pg
from pymoto_gb300.core import HOST_RUNTIME, Module, Network, Signal


class Square(Module):
    def __call__(self, x):
        self.x = x
        return x ** 2

    def _sensitivity(self, dy):
        return 2 * self.x * dy


class Sum(Module):
    def __call__(self, x):
        self.n = x.size
        return float(np.sum(x))

    def _sensitivity(self, df):
        return np.full(self.n, float(df))


class WrongScale(Module):
    """y = 3 x with a sensitivity of 2 dy: every entry must fail."""

    def __call__(self, x):
        return 3.0 * x

    def _sensitivity(self, dy):
        return 2.0 * dy


class Mix(Module):
    """y = [a x0 x1, x2 / a] with a scalar input a."""

    def __call__(self, x, a):
        self.x, self.a = x, a
        return np.array([a * x[0] * x[1], x[2] / a])

    def _sensitivity(self, dy):
        x, a = self.x, self.a
        dx = np.array([a * x[1] * dy[0], a * x[0] * dy[0], dy[1] / a])
        da = x[0] * x[1] * dy[0] - x[2] / a ** 2 * dy[1]
        return dx, da


def test_correct_sensitivities_pass(capsys):
    np.random.seed(0)
    sx = Signal("x", np.random.rand(6) + 0.5)
    with Network() as fn:
        sy = Square()(sx)
        sc = Sum()(sy)
    out = pg.finite_difference(sx, sc, fn, dx=1e-6, tol=1e-5, verbose=False)
    assert out == {"x": (0, 6)}
    out = pg.finite_difference(sx, sc, fn, dx=1e-4, tol=1e-7, verbose=False, central=True, entries=[0, 3, 99])
    assert out == {"x": (0, 2)}


def test_wrong_sensitivities_are_reported(capsys):
    np.random.seed(1)
    sx = Signal("x", np.random.rand(5) + 0.1)
    with Network() as fn:
        sy = WrongScale()(sx)
    out = pg.finite_difference(sx, sy, fn, dx=1e-6, verbose=False)
    assert out == {"x": (5, 5)}
    assert "<--*" in capsys.readouterr().out


def test_vector_output_scalar_input_and_zero_structure(capsys):
    np.random.seed(2)
    sx = Signal("x", np.array([0.7, 0.0, 1.3]))
    sa = Signal("a", 2.5)
    with Network() as fn:
        sy = Mix()(sx, sa)
    out = pg.finite_difference([sx, sa], sy, fn, dx=1e-7, tol=1e-5, verbose=False)
    assert out == {"x": (0, 2), "a": (0, 1)}          # x[1] == 0 is skipped (keep_zero_structure)
    out = pg.finite_difference([sx, sa], sy, fn, dx=1e-7, tol=1e-5, verbose=False, keep_zero_structure=False)
    assert out == {"x": (0, 3), "a": (0, 1)}
    assert sx.state[1] == 0.0 and sa.state == 2.5          # inputs restored


@pytest.mark.skipif(HOST_RUNTIME != "standalone", reason="the standalone runtime's network helpers")
def test_network_cones_and_stub_signals():
    sx, sz = Signal("x", np.ones(3)), Signal("z", np.ones(2))
    with Network() as fn:
        sy = Square()(sx)
        sc = Sum()(sy)
        sw = Square()(sz)                                  # unrelated branch
    assert set(fn.sig_in) == {sx, sz} and set(fn.sig_out) == {sc, sw}
    cone = fn.get_output_cone(sc)
    assert [type(m).__name__ for m in cone] == ["Square", "Sum"] and cone.sig_in == [sx]
    assert len(fn.get_input_cone(sz)) == 1 and fn.get_input_cone(sz).sig_out == [sw]
    assert len(fn.get_output_cone(sc).get_input_cone(sz)) == 0
    with pytest.raises(RuntimeError):
        pg.finite_difference(sz, sc, fn)


@pytest.mark.gpu
def test_finite_difference_on_the_device_network(capsys):
    """The compliance network with a device design: central differences (h = 1e-4 x) on 16 seeded elements,
    the same check as the pipeline's own finite-difference test, through finite_difference."""
    import torch
    import oracle as O
    from conftest import clamp_face_dofs
    from test_gpu_pipeline import build_network
    shape = (16, 8, 8)
    g = O.Grid(*shape)
    bc = clamp_face_dofs(g)
    f = np.zeros(g.ndof)
    f[3 * g.node_number(16, 4, 4) + 1] = -1.0
    _, sx, _, sc, fn = build_network(pg, shape, bc, f, "conv", 2.5, 3, 1e-12, state_kind="torch")
    rng = np.random.default_rng(5)
    sx.state = torch.from_numpy(rng.uniform(0.1, 1.0, g.nel)).cuda()
    els = rng.choice(g.nel, 16, replace=False)
    out = pg.finite_difference(sx, sc, fn, dx=1e-4, relative_dx=True, tol=1e-5, use_df=[1.0], verbose=False,
                               entries=els, central=True)
    assert out == {"x": (0, 16)}


def test_optimizer_slice_network_keeps_only_the_connecting_modules():
    sx, sz = Signal("x", np.ones(3)), Signal("z", np.ones(2))
    with Network() as fn:
        sy = Square()(sx)
        sc = Sum()(sy)
        Square()(sz)
    oc = pg.OC(sx, sc, fn, slice_network=True, verbosity=0)
    assert [type(m).__name__ for m in oc.function] == ["Square", "Sum"]
    with pytest.raises(RuntimeError):
        pg.OC(sz, sc, fn, slice_network=True)
