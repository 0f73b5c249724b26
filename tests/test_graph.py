"""Standalone graph runtime: pyMOTO's Signal / Module / Network protocol (no GPU)."""
import numpy as np
import pytest

from pymoto_gb300 import _graph as G


class Square(G.Module):
    def __call__(self, x):
        return x * x

    def _sensitivity(self, dy):
        return 2 * self.get_input_states() * dy


class Mul(G.Module):
    def __call__(self, a, b):
        return a * b

    def _sensitivity(self, dy):
        a, b = self.get_input_states()
        return dy * b, dy * a


def test_network_response_and_reverse_sweep():
    sx = G.Signal("x", np.array([1.0, 2.0, 3.0]))
    with G.Network() as fn:
        sy = Square()(sx)
        sz = Mul()(sy, sx)      # z = x^3
    assert len(fn) == 2
    np.testing.assert_allclose(sz.state, [1, 8, 27])
    sx.state = np.array([2.0, 3.0, 4.0])
    fn.response()
    np.testing.assert_allclose(sz.state, [8, 27, 64])
    sz.sensitivity = np.ones(3)
    fn.sensitivity()
    np.testing.assert_allclose(sx.sensitivity, 3 * sx.state ** 2)   # two contributions accumulated
    fn.reset()
    assert sx.sensitivity is None


def test_add_sensitivity_deep_copies_first_contribution():
    s = G.Signal("a")
    d = np.ones(2)
    s.add_sensitivity(d)
    s.add_sensitivity(d)
    np.testing.assert_allclose(s.sensitivity, 2.0)
    np.testing.assert_allclose(d, 1.0)


def test_keyword_only_arguments_rejected():
    with pytest.raises(SyntaxError):
        class Bad(G.Module):
            def __call__(self, x, *, y=1):
                return x


def test_module_added_to_active_networks_once():
    sx = G.Signal("x", 1.0)
    with G.Network() as fn:
        m = Square()
        m(sx)
        with pytest.raises(RuntimeError):
            m(sx)
    assert fn.mods == [m]


def test_constant_inputs_give_plain_values():
    assert Square()(3.0) == 9.0


def test_add_sensitivity_copies_tensors_with_clone():
    """A tensor's first contribution is copied (clone), so later in-place accumulation leaves the producer's
    tensor untouched."""
    torch = pytest.importorskip("torch")
    s = G.Signal("s")
    first = torch.ones(4)
    s.add_sensitivity(first)
    s.add_sensitivity(torch.ones(4))
    assert torch.equal(s.sensitivity, torch.full((4,), 2.0)) and torch.equal(first, torch.ones(4))


def test_hierarchy_per_level_coarse_smoothing():
    """coarse_smooth_steps as a list: one value per level below the finest, the last one repeated."""
    import pymoto_gb300 as pg
    d = pg.VoxelDomain(32, 16, 16)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=5, smooth_steps=1, coarse_smooth_steps=[2, 3],
                                          smoother="chebyshev")
    assert [m.smooth_steps for m in mgs] == [1, 2, 3, 3]
    assert [m.smoother.degree for m in mgs] == [1, 2, 3, 3]


def test_hierarchy_construction_without_a_gpu():
    """Level count (given, or automatic down to max_coarse_dofs), sub-domains with doubled element sizes, the
    lagged coarsest solve, and the errors for grids that do not halve."""
    import pymoto_gb300 as pg
    d = pg.VoxelDomain(128, 64, 64, 0.5, 0.5, 0.5)
    mgs = pg.GeometricMultigrid.hierarchy(d, levels=5, smoother_w=0.6, smooth_steps=2, coarse_lag=True)
    assert [m.grid.dims for m in mgs] == [(128, 64, 64), (64, 32, 32), (32, 16, 16), (16, 8, 8)]
    assert all(m.inner_level is n for m, n in zip(mgs, mgs[1:]))
    assert isinstance(mgs[-1].inner_level, pg.DenseCholesky) and mgs[-1].inner_level.lag
    assert mgs[1].domain.unitx == 1.0 and mgs[3].sub_domain.unitx == 8.0
    auto = pg.GeometricMultigrid.hierarchy(d, smoother_w=0.6, smooth_steps=2, max_coarse_dofs=3000)
    coarsest = auto[-1].grid.coarse()
    assert coarsest.ndof <= 3000 < auto[-1].grid.ndof
    with pytest.raises(ValueError):
        pg.GeometricMultigrid(pg.VoxelDomain(9, 4, 4))
    with pytest.raises(ValueError):
        pg.GeometricMultigrid.hierarchy(pg.VoxelDomain(12, 6, 6), levels=4)
    with pytest.raises(ValueError):
        pg.GeometricMultigrid.hierarchy(d, smoother="sor")
