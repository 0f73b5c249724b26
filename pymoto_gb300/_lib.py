"""ctypes binding of libpymoto_gb300.so (the C ABI of include/pymoto_gb300.h).

There is no CPU fallback: if the library cannot be loaded, every operation raises.
"""
import ctypes
import os
import threading
from ctypes import c_char_p, c_double, c_float, c_int, c_int64, c_size_t, c_void_p

import numpy as np
import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpymoto_gb300.so")

P = c_void_p
I = c_int
D = c_double
L = c_int64
F = c_float

# name -> (restype, argtypes); mirrors include/pymoto_gb300.h
SIGNATURES = {
    "pmg_version": (I, []),
    "pmg_status_string": (c_char_p, [I]),
    "pmg_last_error": (c_char_p, []),
    "pmg_element_stiffness": (I, [I, D, D, I, D, D, D, P]),
    "pmg_dof_connectivity": (I, [I, I, I, P, P]),
    "pmg_ebe_apply": (I, [I, I, I, I, I, P, P, P, D, P, P, P, D, P, P, P]),
    "pmg_ebe_diagonal": (I, [I, I, I, I, P, P, P, D, P, P, P]),
    "pmg_stencil_apply": (I, [I, I, I, I, I, P, P, P, P, D, P, P]),
    "pmg_stencil_diagonal": (I, [I, I, I, I, P, P, P]),
    "pmg_stencil_add_diagonal": (I, [I, I, I, I, P, P, P]),
    "pmg_restrict": (I, [I, I, I, I, P, P, P]),
    "pmg_prolong_add": (I, [I, I, I, I, P, P, P]),
    "pmg_galerkin_table": (I, [I, P, P]),
    "pmg_galerkin_from_ebe": (I, [I, I, I, I, P, P, P, D, P, P, I, P, P]),
    "pmg_galerkin_from_elements": (I, [I, I, I, I, P, P, P]),
    "pmg_stencil_from_elements": (I, [I, I, I, I, P, P, P]),
    "pmg_stencil_to_dense": (I, [I, I, I, I, P, P, P]),
    "pmg_stencil_to_dense_perm": (I, [I, I, I, I, P, P, P, P]),
    "pmg_coarse_ordering": (I, [I, I, I, P, P]),
    "pmg_ebe_stencil": (I, [I, I, I, I, P, P, P, D, P, P]),
    "pmg_stencil_bandwidth": (I, [I, I, I]),
    "pmg_stencil_rowabs": (I, [I, I, I, I, P, P, P]),
    "pmg_cheb_coeffs": (I, [P, D, D, I, P, P]),
    "pmg_cheb_step": (I, [I, L, P, P, P, P, P, I, I, P]),
    "pmg_stencil_cheb_step": (I, [I, I, I, I, P, P, P, P, P, P, I, P, P]),
    "pmg_ebe_cheb_step": (I, [I, I, I, P, P, P, D, P, P, P, P, P, I, P, P, P]),
    "pmg_operator_status": (I, [I]),
    "pmg_set_operator_kernel": (I, [I]),
    "pmg_set_wait_test": (I, [ctypes.c_uint, I]),
    "pmg_cholesky_factor": (I, [I, P, I, P, P]),
    "pmg_cholesky_solve": (I, [I, I, P, I, P, P, P]),
    "pmg_cholesky_inverse": (I, [I, P, I, P, P]),
    "pmg_cholesky_block_inverses": (I, [I, I, P, P, P]),
    "pmg_cholesky_solve_blocked": (I, [I, I, P, I, P, P, P, P]),
    "pmg_cholesky_inverse_f32_scratch_bytes": (c_size_t, [I]),
    "pmg_cholesky_inverse_f32": (I, [I, P, I, P, P, P]),
    "pmg_dense_gemv": (I, [I, I, P, P, P, P]),
    "pmg_dense_permute": (I, [I, I, P, P, P, P]),
    "pmg_reduce_scratch_bytes": (c_size_t, []),
    "pmg_dot": (I, [I, L, P, P, P, P, P]),
    "pmg_dot2": (I, [I, L, P, P, P, P, P, P, P]),
    "pmg_dot_noalloc": (I, [I, L, P, P, P, P]),
    "pmg_cg_update": (I, [I, L, P, P, P, P, P, P, P, P, P]),
    "pmg_axpy_ratio": (I, [I, L, P, P, P, P, D, P]),
    "pmg_xpby_ratio": (I, [I, L, P, P, P, P, P]),
    "pmg_scale_rsqrt": (I, [I, L, P, P, P, P]),
    "pmg_scale": (I, [I, L, P, P, D, P]),
    "pmg_mask_bc": (I, [I, I, L, P, I, P, P, P]),
    "pmg_split_bc": (I, [I, I, L, P, D, P, P, P, P, P]),
    "pmg_convert": (I, [I, I, L, P, P, D, P]),
    "pmg_add_f32_to_f64": (I, [L, P, P, D, P]),
    "pmg_convert_dscale": (I, [I, I, L, P, P, P, I, P]),
    "pmg_diag_scale": (I, [I, L, P, P, D, P, P]),
    "pmg_density_filter_rowsum": (I, [I, I, I, D, P, P]),
    "pmg_density_filter": (I, [I, I, I, I, D, P, P, P, P]),
    "pmg_conv_filter": (I, [I, I, I, P, I, I, I, P, P, P, P, P, P]),
    "pmg_conv_filter_adjoint": (I, [I, I, I, P, I, I, I, P, P, P, P, P, P, P, P, P]),
    "pmg_simp": (I, [L, D, D, P, P, P, P]),
    "pmg_simp_backward": (I, [L, D, D, P, P, P, P]),
    "pmg_sens_contract": (I, [I, I, I, P, P, P, P, D, I, P, P]),
    "pmg_sens_contract_mixed": (I, [I, I, I, P, P, P, P, D, I, P, P]),
    "pmg_oc_scratch_bytes": (c_size_t, []),
    "pmg_oc_status": (I, [P]),
    "pmg_oc_status_async": (I, [P, P, P]),
    "pmg_oc_update": (I, [L, P, P, P, D, D, D, D, D, D, D, P, P]),
    "pmg_overhang_forward": (I, [I] * 13 + [P] + [D] * 5 + [P] * 4),
    "pmg_overhang_adjoint": (I, [I] * 14 + [P] + [D] * 5 + [P] * 8),
    "pmg_mma_scratch_bytes": (c_size_t, [L, I]),
    "pmg_mma_update": (I, [L] + [P] * 16),
    "pmg_nn_conv3d_forward": (I, [I, I, I, I, I, I, P, P, P, I, P, P, P]),
    "pmg_nn_conv3d_backward_data": (I, [I, I, I, I, I, P, P, P, P]),
    "pmg_nn_wgrad_scratch_bytes": (c_size_t, [I, I, I, I, I]),
    "pmg_nn_conv3d_backward_weights": (I, [I, I, I, I, I, I, P, P, P, I, P, P]),
    "pmg_nn_relu_backward": (I, [L, P, P, P]),
    "pmg_nn_pool2": (I, [I, I, I, I, I, P, P, P]),
    "pmg_nn_up2": (I, [I, I, I, I, I, I, I, P, P, P]),
    "pmg_nn_copy_channels": (I, [L, I, I, I, P, P, P]),
    "pmg_nn_split_channels": (I, [L, I, I, I, P, P, P]),
    "pmg_nn_input_features": (I, [I, I, I, I, I, I, I, P, P, P]),
    "pmg_nn_vox_to_node": (I, [I, I, I, I, P, P, P]),
    "pmg_nn_adam": (I, [I, P, P, P, P, P, F, F, F, F, I, F, P]),
    "pmg_nn_mse": (I, [L, P, P, D, P, P, P]),
    "pmg_nn_inject": (I, [I, I, I, I, P, D, P, P]),
    "pmg_scalar_stencil": (I, [I, I, I, I, P, P, P, D, P, P, P]),
    "pmg_scalar_apply": (I, [I, I, I, I, I, P, P, P, P, D, P, P]),
    "pmg_scalar_restrict": (I, [I, I, I, I, P, P, P]),
    "pmg_scalar_prolong_add": (I, [I, I, I, I, P, P, P]),
    "pmg_scalar_galerkin": (I, [I, I, I, I, P, P, P]),
    "pmg_scalar_to_dense": (I, [I, I, I, I, P, P, P]),
    "pmg_scalar_rowabs": (I, [I, I, I, I, P, P, P]),
    "pmg_scalar_sens": (I, [I, I, I, P, P, P, P, D, I, P, P]),
    "pmg_operator_plan": (I, [I, I, I, I, P]),
}

# Returns that are values, not statuses
_VALUE_RETURNING = {"pmg_version", "pmg_status_string", "pmg_last_error", "pmg_reduce_scratch_bytes",
                    "pmg_oc_scratch_bytes", "pmg_stencil_bandwidth", "pmg_mma_scratch_bytes",
                    "pmg_set_operator_kernel"}

F64, F32 = 0, 1
MATVEC, RESIDUAL, JACOBI = 0, 1, 2


class PMGError(RuntimeError):
    """A pymoto_gb300 C-ABI call returned a non-zero status."""

    def __init__(self, name, status, detail=""):
        self.status = status
        super().__init__(f"{name} failed with status {status}{': ' + detail if detail else ''}")


_lib = None
_lock = threading.Lock()


def load():
    """Load the CUDA library, building it first when it is absent (nvcc required)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from .build import build
            build()
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def _arg(a):
    if a is None:
        return None
    if type(a) is torch.Tensor or isinstance(a, torch.Tensor):
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if isinstance(a, bool):
        return int(a)
    return a


# kernels launched per call where it is not exactly one (host-only entry points launch none)
_HOST_ONLY = {"pmg_version", "pmg_status_string", "pmg_last_error", "pmg_element_stiffness", "pmg_galerkin_table",
              "pmg_reduce_scratch_bytes", "pmg_oc_scratch_bytes", "pmg_stencil_bandwidth",
              "pmg_cholesky_inverse_f32_scratch_bytes", "pmg_nn_wgrad_scratch_bytes", "pmg_oc_status",
              "pmg_coarse_ordering", "pmg_oc_status_async", "pmg_mma_scratch_bytes", "pmg_operator_status",
              "pmg_set_wait_test", "pmg_set_operator_kernel", "pmg_operator_plan"}


def _launches(name, args):
    if name in _HOST_ONLY:
        return 0
    if name == "pmg_cholesky_factor":
        return 1          # one thread-block cluster for the whole factorisation
    if name == "pmg_cholesky_inverse_f32":
        return 4
    if name == "pmg_galerkin_from_ebe":
        return 2 if args[9] is not None and int(args[10]) > 0 else 1
    if name in ("pmg_nn_conv3d_backward_weights", "pmg_scalar_galerkin"):
        return 2          # weight partials + their sum; forward offsets + the mirrored backward ones
    if name == "pmg_mma_update":
        return 3          # reset, the cooperative solve, status
    if name == "pmg_oc_update":
        # init + one cooperative launch while the design fits the registers of the resident CTAs (2 CTAs of
        # 256 threads x 8 elements per SM); above that init + prepare + one launch per step + final
        if int(args[0]) <= 152 * 2 * 256 * 8:
            return 2
        width, steps = float(args[9]) - float(args[8]), 3
        while width > float(args[10]):
            width *= 0.5
            steps += 1
        return steps
    return 1


class Probe:
    """Counts kernel launches and, for the entry points in `targets` (None = all), brackets each call with
    CUDA events on the launching stream.  Use as a context manager; `summary()` after synchronising."""

    active = None

    def __init__(self, targets=None, key_args=3):
        self.targets = targets
        self.key_args = key_args
        self.launches = 0
        self.records = []

    def __enter__(self):
        Probe.active = self
        return self

    def __exit__(self, *exc):
        Probe.active = None

    def replay(self, key, graph, launches):
        """Replay a captured CUDA graph; counted and (when `targets` is None or contains "graph") timed."""
        self.launches += launches
        if self.targets is None or "graph" in self.targets:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            graph.replay()
            e1.record()
            self.records.append((("graph", key), e0, e1))
        else:
            graph.replay()

    def summary(self):
        out = {}
        for key, e0, e1 in self.records:
            d = out.setdefault(key, [0, 0.0])
            d[0] += 1
            d[1] += e0.elapsed_time(e1)
        return {k: {"launches": v[0], "total_ms": v[1], "avg_ms": v[1] / v[0]} for k, v in out.items()}


def replay(key, graph, launches):
    """Replay a CUDA graph of library kernels (accounted to the active Probe, if any)."""
    if Probe.active is not None:
        Probe.active.replay(key, graph, launches)
    else:
        graph.replay()


_fns = {}


def call(name, *args):
    """Call a C-ABI function; raise PMGError on a non-zero status."""
    fn = _fns.get(name)
    if fn is None:
        fn = _fns[name] = getattr(load(), name)
    lib = _lib
    pr = Probe.active
    if pr is not None:
        pr.launches += _launches(name, args)
        if pr.targets is None or name in pr.targets:
            if name not in _HOST_ONLY:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                rc = fn(*[_arg(a) for a in args])
                e1.record()
                key = (name,) + tuple(a for a in args[:pr.key_args] if isinstance(a, int))
                pr.records.append((key, e0, e1))
            else:
                rc = fn(*[_arg(a) for a in args])
        else:
            rc = fn(*[_arg(a) for a in args])
    else:
        rc = fn(*[_arg(a) for a in args])
    if name in _VALUE_RETURNING:
        return rc
    if rc != 0:
        msg = lib.pmg_status_string(rc).decode()
        err = lib.pmg_last_error().decode()
        raise PMGError(name, rc, msg + (f" ({err})" if err else ""))
    return rc


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)
_cur_device = getattr(torch._C, "_cuda_getDevice", None)


def stream():
    """Handle of the current torch CUDA stream (all library calls are ordered on it).  Read through torch's
    raw-handle accessor where it exists: torch.cuda.current_stream() builds a Stream object per call, which
    is most of the host cost of a small library call."""
    if _raw_stream is not None and _cur_device is not None:
        return _raw_stream(_cur_device())
    return torch.cuda.current_stream().cuda_stream


def dtype_code(t):
    if t.dtype == torch.float64:
        return F64
    if t.dtype == torch.float32:
        return F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def require_cuda(t, name="tensor"):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
        raise TypeError(f"{name} must be a contiguous CUDA tensor")
    return t
