"""MathExpression against pyMOTO's MathExpression on the same inputs: numpy states (pyMOTO's evaluation), torch
CPU tensors (the torch function table and the reverse broadcasting on tensors), and CUDA tensors (GPU)."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

import pymoto_gb300 as pg
from pymoto_gb300.core import Signal


def _cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.math_cases()


NAMES = [c[0] for c in _cases()]


def _run(case, conv):
    name, expr, tags, inputs, seed = next(c for c in _cases() if c[0] == case)
    sigs = [Signal(t, conv(v)) for t, v in zip(tags, inputs)]
    m = pg.MathExpression(expr)
    so = m(*sigs)
    return so.state, m._sensitivity(conv(seed))


def _host(v):
    return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)


def _check(case, y, ds, golden):
    g = golden("math_expression.npz")
    np.testing.assert_allclose(_host(y), g[f"{case}_y"], rtol=1e-14, atol=1e-15)
    for i, d in enumerate(ds):
        np.testing.assert_allclose(_host(d), g[f"{case}_d{i}"], rtol=1e-14, atol=1e-15)
        assert np.shape(_host(d)) == np.shape(g[f"{case}_d{i}"])


@pytest.mark.parametrize("case", NAMES)
def test_numpy_states_match_pymoto(case, golden):
    y, ds = _run(case, lambda v: v)
    _check(case, y, ds, golden)


@pytest.mark.parametrize("case", NAMES)
def test_torch_states_match_pymoto(case, golden):
    def conv(v):   # the SIMP case's input is a scalar: the generic path (the SIMP kernels take element fields)
        return torch.as_tensor(np.asarray(v, dtype=np.float64))
    y, ds = _run(case, conv)
    _check(case, y, ds, golden)


def test_duplicate_names_are_rejected():
    with pytest.raises(RuntimeError):
        a, b = Signal("inp1", 1.0), Signal("y", 2.0)
        pg.MathExpression("inp1 + y")(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("case", NAMES)
def test_device_states_match_pymoto(case, golden):
    y, ds = _run(case, lambda v: torch.as_tensor(np.asarray(v, dtype=np.float64)).cuda())
    _check(case, y, ds, golden)


@pytest.mark.parametrize("text,xmin,penal", [("1e-9 + (1-1e-9)*inp0^3", 1e-9, 3.0),
                                             ("0.001+(1-0.001)*inp0**3.5", 1e-3, 3.5)])
def test_simp_form_selects_the_simp_kernels(text, xmin, penal):
    m = pg.MathExpression(text)
    assert m._simp is not None and (m.xmin, m.penal) == (xmin, penal)


@pytest.mark.parametrize("text", ["1e-9 + (1-1e-3)*inp0^3", "inp0^3", "1e-9 + (1-1e-9)*inp0^3 + inp1"])
def test_other_expressions_are_not_taken_for_simp(text):
    assert pg.MathExpression(text)._simp is None
