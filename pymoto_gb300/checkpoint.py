"""Checkpoint and resume of a design run: design signals, optimizer state (OC, MMA), the solver's warm start
(LinSolve) and the learned warm start (network weights, Adam moments, training buffer, its random state).

save_checkpoint(path, **objects) writes one .npz (no pickling): every object's state_dict() under its name,
tensors copied to the host (BF16 tensors stored as their 16-bit patterns), Python scalars and structures as
JSON.  load_checkpoint(path, **objects) restores them in place, device tensors back on the device they were
built for.  With the FP64 solver path the next design iteration after a resume reproduces the uninterrupted
run's compliance bit for bit (the kernels and reductions are deterministic); the mixed path's lagged coarse
inverse is rebuilt, so its first solve after a resume may take a different number of iterations.
"""
import json

import numpy as np
import torch


def _pack(prefix, value, arrays, meta):
    if isinstance(value, torch.Tensor):
        t = value.detach()
        if t.dtype == torch.bfloat16:
            arrays[prefix] = t.view(torch.int16).cpu().numpy()
            meta[prefix] = {"kind": "tensor", "dtype": "bfloat16", "cuda": t.is_cuda}
        else:
            arrays[prefix] = t.cpu().numpy()
            meta[prefix] = {"kind": "tensor", "cuda": t.is_cuda}
    elif isinstance(value, np.ndarray):
        arrays[prefix] = value
        meta[prefix] = {"kind": "ndarray"}
    elif isinstance(value, (list, tuple)) and any(isinstance(v, (torch.Tensor, np.ndarray)) for v in value):
        meta[prefix] = {"kind": "list", "n": len(value)}
        for i, v in enumerate(value):
            _pack(f"{prefix}#{i}", v, arrays, meta)
    elif isinstance(value, dict):
        meta[prefix] = {"kind": "dict", "keys": list(value)}
        for k, v in value.items():
            _pack(f"{prefix}.{k}", v, arrays, meta)
    else:
        meta[prefix] = {"kind": "json", "value": value if not isinstance(value, np.generic) else value.item()}


def _unpack(prefix, arrays, meta, device):
    m = meta[prefix]
    kind = m["kind"]
    if kind == "tensor":
        a = arrays[prefix]
        t = torch.from_numpy(np.array(a))
        if m.get("dtype") == "bfloat16":
            t = t.view(torch.bfloat16)
        return t.to(device) if m["cuda"] and device is not None else t
    if kind == "ndarray":
        return np.array(arrays[prefix])
    if kind == "list":
        return [_unpack(f"{prefix}#{i}", arrays, meta, device) for i in range(m["n"])]
    if kind == "dict":
        return {k: _unpack(f"{prefix}.{k}", arrays, meta, device) for k in m["keys"]}
    return m["value"]


def signal_state(sig):
    return {"state": sig.state}


def save_checkpoint(path, **objects):
    """objects: name -> an object with state_dict() or a Signal (its state is saved)."""
    arrays, meta = {}, {}
    for name, obj in objects.items():
        sd = obj.state_dict() if hasattr(obj, "state_dict") else signal_state(obj)
        _pack(name, sd, arrays, meta)
    arrays["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez(path, **arrays)


def load_checkpoint(path, device=None, **objects):
    """Restore the objects saved under the same names; `device` for CUDA tensors (default: the current one)."""
    if device is None and torch.cuda.is_available():
        device = torch.device("cuda", torch.cuda.current_device())
    with np.load(path, allow_pickle=False) as f:
        arrays = {k: f[k] for k in f.files}
    meta = json.loads(bytes(arrays.pop("__meta__")).decode())
    for name, obj in objects.items():
        sd = _unpack(name, arrays, meta, device)
        if hasattr(obj, "load_state_dict"):
            obj.load_state_dict(sd)
        else:
            obj.state = sd["state"]
