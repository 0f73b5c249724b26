"""EinSum for any expression against pyMOTO's EinSum (tests/golden/einsum.npz): numpy states and torch
tensors on the CPU; device tensors on the GPU.  The compliance-path forms 'i,i->' and 'i->' run in the FP64
dot kernel and are covered by the pipeline tests."""
import numpy as np
import pytest
import torch

import pymoto_gb300 as pg
from pymoto_gb300.core import Signal

EXPRS = ["i,i->i", "i,j->ij", "ii->", "ij,j->i", "i,ij,j->", "ij,ij->ij", "ji,ij->ij", "ji,jk,kl->il", "ij->",
         "ijk,k->ij"]


def _case(n, golden):
    g = golden("einsum.npz")
    args = []
    i = 0
    while f"e{n}_a{i}" in g:
        args.append(g[f"e{n}_a{i}"])
        i += 1
    return g, args


def _run(n, golden, conv):
    g, args = _case(n, golden)
    m = pg.EinSum(EXPRS[n])
    y = m(*[Signal(f"a{i}", conv(a)) for i, a in enumerate(args)]).state
    ds = m._sensitivity(conv(g[f"e{n}_dy"]))
    ds = ds if isinstance(ds, list) else [ds]
    to_np = lambda v: v.cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)  # noqa: E731
    np.testing.assert_allclose(to_np(y), g[f"e{n}_y"], rtol=1e-13, atol=1e-14)
    assert len(ds) == len(args)
    for i, d in enumerate(ds):
        np.testing.assert_allclose(to_np(d), g[f"e{n}_d{i}"], rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("n", range(len(EXPRS)), ids=EXPRS)
def test_numpy_states_match_pymoto(n, golden):
    _run(n, golden, lambda a: a)


@pytest.mark.parametrize("n", range(len(EXPRS)), ids=EXPRS)
def test_torch_states_match_pymoto(n, golden):
    _run(n, golden, lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64)))


def test_repeated_indices_need_the_scalar_form():
    m = pg.EinSum("ii->i")
    m(Signal("A", np.eye(3)))
    with pytest.raises(NotImplementedError):
        m._sensitivity(np.ones(3))


@pytest.mark.gpu
@pytest.mark.parametrize("n", range(len(EXPRS)), ids=EXPRS)
def test_device_states_match_pymoto(n, golden):
    _run(n, golden, lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64)).cuda())
