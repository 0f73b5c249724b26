"""ScalarToFile against the logs pyMOTO's ScalarToFile wrote for the same signals (byte for byte)."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

from pymoto_gb300 import Network, ScalarToFile, Signal


def _cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.scalar_cases()


def _run(tmp_path, fname, fmt, sep, its, convert=lambda v: v):
    out = str(tmp_path / "log" / fname)
    sigs = [Signal(tag, convert(val)) for tag, val in its[0].items()]
    with Network() as fn:
        m = ScalarToFile(out, fmt=fmt, separator=sep)
        m(*sigs)
    for vals in its[1:]:
        for s in sigs:
            s.state = convert(vals[s.tag])
        fn.response()
    m.flush()
    with open(out, "rb") as f:
        return f.read()


def _golden(fname):
    with open(os.path.join(GOLDEN, fname), "rb") as f:
        return f.read()


@pytest.mark.parametrize("case", [c[0] for c in _cases()])
def test_log_matches_pymoto(case, tmp_path):
    name, fname, fmt, sep, its = next(c for c in _cases() if c[0] == case)
    assert _run(tmp_path, fname, fmt, sep, its) == _golden(fname)


def test_log_from_torch_cpu_tensors(tmp_path):
    name, fname, fmt, sep, its = _cases()[0]
    conv = lambda v: torch.as_tensor(v) if isinstance(v, np.ndarray) else v  # noqa: E731
    assert _run(tmp_path, fname, fmt, sep, its, conv) == _golden(fname)


def test_rejects_bad_format_and_non_signals(tmp_path):
    with pytest.raises(ValueError):
        ScalarToFile(str(tmp_path / "a.txt"), fmt="not-a-format")
    with pytest.raises(NotImplementedError):      # constants, not signals: pyMOTO raises the same
        ScalarToFile(str(tmp_path / "b.txt"))(1.0)


@pytest.mark.gpu
def test_log_from_device_scalars(tmp_path):
    """Responses as CUDA tensors (0-d and vectors): the same bytes, no synchronisation in the call."""
    name, fname, fmt, sep, its = _cases()[0]

    def conv(v):
        if isinstance(v, (float, np.floating)):
            return torch.tensor(float(v), dtype=torch.float64, device="cuda")
        if isinstance(v, np.ndarray):
            return torch.as_tensor(v).cuda()
        return v
    assert _run(tmp_path, fname, fmt, sep, its, conv) == _golden(fname)
