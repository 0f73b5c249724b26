"""pmg_dot_noalloc, the dot product for callers that cannot allocate device memory (GPU).

Some callers of this library cannot call cudaMalloc -- for example a plugin inside a host application that
owns every device allocation.  pmg_dot_noalloc keeps its reduction scratch in a static device array, so such
a caller passes only inputs and output.  This file is collected last on purpose: it runs after every other
test in a full run, and also passes when run alone in a fresh process.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from pymoto_gb300 import _lib
    _lib.load()
    return _lib


@pytest.mark.parametrize("n", [0, 1, 1000, 1_635_075, 4_194_304])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_dot_matches_pmg_dot_twice_in_a_row(lib, n, dtype):
    from pymoto_gb300.operators import Workspace
    rng = np.random.default_rng(n + 7)
    # buffers of at least one element: an empty tensor has a null data pointer, which both entry points reject
    a = torch.from_numpy(rng.standard_normal(max(n, 1))).to("cuda", dtype)
    b = torch.from_numpy(rng.standard_normal(max(n, 1))).to("cuda", dtype)
    code = lib.F64 if dtype == torch.float64 else lib.F32
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib.call("pmg_dot", code, n, a, b, ref, Workspace.get().reduce, lib.stream())
    outs = []
    for _ in range(2):   # two calls in a row share the static scratch
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        lib.call("pmg_dot_noalloc", code, n, a, b, out, lib.stream())
        outs.append(out.item())
    r = ref.item()
    scale = max(1.0, abs(r))
    for v in outs:
        assert abs(v - r) <= 1e-12 * np.sqrt(max(n, 1)) * scale, (v, r)
    assert outs[0] == outs[1]


def test_noalloc_dot_rejects_n_beyond_its_scratch(lib):
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(lib.PMGError) as e:
        lib.call("pmg_dot_noalloc", lib.F64, 4_194_305, a, a, out, lib.stream())
    assert e.value.status == 1
    assert "4194304" in str(e.value)
