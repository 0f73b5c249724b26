"""VTI output against the files pyMOTO's VoxelDomain.write_to_vti wrote for the same inputs (byte for byte)."""
import importlib.util
import os
import warnings

import numpy as np
import pytest
import torch

from conftest import GOLDEN

from pymoto_gb300 import Network, Signal, VoxelDomain
from pymoto_gb300 import vti


def _cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.vti_cases()


def _domain(shp, size, origin):
    d = VoxelDomain(*shp, *size)
    d.origin = np.array(origin)
    return d


def _golden(name):
    with open(os.path.join(GOLDEN, f"vti_{name}.vti"), "rb") as fh:
        return fh.read()


@pytest.mark.parametrize("case", [c[0] for c in _cases()])
def test_vti_bytes_match_pymoto(case, tmp_path):
    name, shp, size, origin, scale, vecs = next(c for c in _cases() if c[0] == case)
    d = _domain(shp, size, origin)
    fn = str(tmp_path / "out")                         # the extension is appended, as in pyMOTO
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        d.write_to_vti(vecs, filename=fn, scale=scale)
    assert (name != "h8") or any("bad" in str(x.message) for x in w)
    with open(fn + ".vti", "rb") as fh:
        assert fh.read() == _golden(name)


def test_vti_torch_cpu_tensors_and_async(tmp_path):
    name, shp, size, origin, scale, vecs = _cases()[1]
    d = _domain(shp, size, origin)
    tv = {k: torch.as_tensor(v) for k, v in vecs.items()}
    t = vti.write_to_vti(d, tv, str(tmp_path / "a.vti"), scale)
    vti.flush()
    assert not t.is_alive()
    assert (tmp_path / "a.vti").read_bytes() == _golden(name)


def test_vti_nothing_to_write(tmp_path):
    d = VoxelDomain(3, 2)
    with pytest.warns(UserWarning):
        assert vti.encode_vti(d, {"bad": np.zeros(5)}) is None


def test_write_to_vti_module_numbering(tmp_path):
    d = VoxelDomain(4, 3, 2)
    sx = Signal("x", np.linspace(0, 1, d.nel))
    with Network() as fn:
        m = vti.WriteToVTI(d, saveto=str(tmp_path / "dat" / "design.vti"), interval=2)
        m(sx)
    for _ in range(3):
        fn.response()
    m.flush()
    files = sorted(os.listdir(tmp_path / "dat"))
    assert files == ["design.0000.vti", "design.0002.vti"]
    data = (tmp_path / "dat" / "design.0000.vti").read_bytes()
    assert data == vti.encode_vti(d, {"x": sx.state})
    assert b'Name="x"' in data
    with pytest.raises(ValueError):
        vti.WriteToVTI(d, saveto=str(tmp_path / "bad.vtu"))


@pytest.mark.gpu
def test_vti_from_device_tensors(tmp_path):
    for name, shp, size, origin, scale, vecs in _cases():
        d = _domain(shp, size, origin)
        dv = {k: torch.as_tensor(v).cuda() for k, v in vecs.items()}
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            d.write_to_vti(dv, filename=str(tmp_path / f"{name}.vti"), scale=scale, wait=False)
            vti.flush()
        assert (tmp_path / f"{name}.vti").read_bytes() == _golden(name)


def test_vti_write_errors_are_reported(tmp_path):
    d = VoxelDomain(3, 2)
    w = vti.VTIWriter()
    w.write(d, {"x": np.zeros(d.nel)}, str(tmp_path / "missing_dir" / "a.vti"))
    with pytest.raises(RuntimeError):
        w.flush()
    w.write(d, {"x": np.zeros(d.nel)}, str(tmp_path / "ok.vti"))
    w.flush()
    assert (tmp_path / "ok.vti").exists()
