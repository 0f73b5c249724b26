"""ScalarToFile against the logs pyMOTO's ScalarToFile wrote for the same signals (byte for byte)."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

import pymoto_gb300 as pg
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


def test_design_log_writes_one_json_line_per_record(tmp_path):
    import json
    import types
    solver = types.SimpleNamespace(iterations=7, last_residual=np.float64(3e-7), fell_back=False,
                                   warm_start=types.SimpleNamespace(predictions=2))
    opt = types.SimpleNamespace(iter=0)
    sc, sv = Signal("c", 12.5), Signal("v", np.array([0.25, 0.5]))
    log = pg.DesignLog(str(tmp_path / "run" / "log.jsonl"), solver=solver, optimizer=opt, compliance=sc, vol=sv)
    for k in range(3):
        opt.iter, sc.state = k, 12.5 - k
        log.record(note="x" * k)
    log.flush()
    rows = [json.loads(line) for line in open(tmp_path / "run" / "log.jsonl")]
    assert [r["iteration"] for r in rows] == [0, 1, 2] and [r["compliance"] for r in rows] == [12.5, 11.5, 10.5]
    assert rows[0]["vol"] == [0.25, 0.5] and rows[2]["note"] == "xx"
    assert rows[0]["iterations"] == 7 and rows[0]["last_residual"] == 3e-7 and rows[0]["learned_predictions"] == 2
    assert rows[0]["fell_back"] is False and all(r["time_s"] >= 0 for r in rows)
