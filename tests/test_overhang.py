"""OverhangFilter against pyMOTO's OverhangFilter: the support cone and smooth parameters of the host side and
the oracle's layer sweep (forward and adjoint, in the per-element form of the kernels) on the CPU; the device
module on the GPU."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

import pymoto_gb300 as pg
from oracle.overhang import overhang_adjoint, overhang_forward


def _cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.overhang_cases()


CASES = {c[0]: c[1:] for c in _cases()}


def _module(name):
    shp, size, direc, ang, ns = CASES[name]
    return pg.OverhangFilter(pg.VoxelDomain(*shp, *size), direction=direc, overhang_angle=ang, nsampling=ns)


@pytest.mark.parametrize("name", list(CASES))
def test_support_cone_matches_pymoto(name, golden):
    g = golden("overhang.npz")
    m = _module(name)
    np.testing.assert_array_equal(m.layer_offsets.shape, g[f"{name}_offsets"].shape)
    np.testing.assert_allclose(m.layer_offsets, g[f"{name}_offsets"], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(m.origin, g[f"{name}_origin"])


@pytest.mark.parametrize("name", list(CASES))
def test_layer_sweep_oracle_matches_pymoto(name, golden):
    g = golden("overhang.npz")
    m = _module(name)
    lay, step = int(np.argmax(np.abs(m.direction))), int(np.sign(m.direction[int(np.argmax(np.abs(m.direction)))]))
    args = (m.grid, m.layer_offsets, m.origin, lay, step, m.p, m.q, m.shift, m.backshift, m.eps)
    y, s = overhang_forward(*args, g[f"{name}_x"])
    np.testing.assert_allclose(y, g[f"{name}_y"], rtol=1e-13, atol=1e-15)
    dx = overhang_adjoint(*args, g[f"{name}_x"], y, s, g[f"{name}_dy"])
    np.testing.assert_allclose(dx, g[f"{name}_dx"], rtol=1e-12, atol=1e-13)


def test_kernel_arguments_checked_before_a_launch():
    from pymoto_gb300._lib import PMGError, call
    good = dict(nx=4, ny=3, nz=1, lay=1, step=1, layer=0, w0=3, w1=1, w2=1, c0=1, c1=1, c2=0, K=2)
    bads = [dict(w0=2), dict(c1=-1), dict(layer=3), dict(lay=3), dict(w1=3), dict(K=0)]
    for bad in bads:
        a = dict(good, **bad)
        with pytest.raises(PMGError):
            call("pmg_overhang_forward", *a.values(), 1, 40.0, 30.0, 1e-3, 1e-3, 1e-4, 1, 2, 3, None)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_device_filter_matches_pymoto(name, golden):
    g = golden("overhang.npz")
    m = _module(name)
    y = m(torch.from_numpy(g[f"{name}_x"]).cuda())
    np.testing.assert_allclose(y.cpu().numpy(), g[f"{name}_y"], rtol=1e-12, atol=1e-14)
    dx = m._sensitivity(torch.from_numpy(g[f"{name}_dy"]).cuda())
    np.testing.assert_allclose(dx.cpu().numpy(), g[f"{name}_dx"], rtol=1e-11, atol=1e-12)
