"""Finite-difference check of module and network sensitivities (pyMOTO's finite_difference,
pymoto/routines.py:12-297), for numpy and device states.

Same signature and the same test as pyMOTO: random (or given) output seeds df, analytic input sensitivities by
one back-propagation per output, then every input entry perturbed by dx (relative to |x| with relative_dx),
the response recomputed and sum(df . (f(x+h) - f(x)) / h) compared with the analytic value at tolerance tol
(relative, or absolute where the analytic value is 0).  Additions for the GPU path, where perturbing all
524,288 entries of a design is not practical: `entries` restricts the perturbation to the given flat indices,
and `central=True` uses (f(x+h) - f(x-h)) / 2h, whose O(h^2) error suits iterative solvers.  Perturbations
and differences of device states stay on the device; only the per-entry scalars are read on the host.
Returns {input tag: (failed, tested)}.
"""
import warnings

import numpy as np
import torch

from .core import Network


def _copy(v):
    if isinstance(v, torch.Tensor):
        return v.detach().clone()
    return v.copy() if hasattr(v, "copy") else v


def _inner(df, dfan):
    """sum(df * dfan) as a Python number (complex where the inputs are)."""
    if isinstance(df, torch.Tensor):
        dfan_t = dfan if isinstance(dfan, torch.Tensor) else torch.as_tensor(np.asarray(dfan), device=df.device)
        return torch.sum(df * dfan_t).item()
    return complex(np.sum(df * dfan)) if np.iscomplexobj(df) or np.iscomplexobj(dfan) else float(np.sum(df * dfan))


def _entry(v, e):
    """Entry e (flat, C order) of an analytic sensitivity, or the value itself for a scalar."""
    if v is None:
        return 0.0
    if isinstance(v, torch.Tensor):
        return v.reshape(-1)[e].item() if v.numel() > 1 else v.reshape(-1)[0].item()
    a = np.asarray(v)
    return a.reshape(-1)[e].item() if a.size > 1 else a.reshape(-1)[0].item()


def _parse(sigs):
    if sigs is None:
        return None
    return list(sigs) if isinstance(sigs, (list, tuple)) else [sigs]


def slice_network(function, variables, responses):
    """The modules between the variables and the responses (Optimizer's slice_network,
    pymoto/common/optimizers.py:55-71); variables without a state are computed first."""
    sub = function.get_output_cone(responses).get_input_cone(variables)
    if len(sub) == 0:
        raise RuntimeError(f"Could not find a network that uses the provided input signals {variables} "
                           f"and produces the requested output signals {responses}")
    for s in variables:
        if s.state is None:
            function.get_output_cone(tosig=s).response()
        if s.state is None:
            raise RuntimeError(f"Input signal {s} has no state.")
    return sub


def finite_difference(fromsig=None, tosig=None, function=None, dx=1e-8, relative_dx=False, tol=1e-5, random=True,
                      use_df=None, test_fn=None, keep_zero_structure=True, verbose=True, entries=None, central=False):
    if function is None:
        function = Network.active[0]
    print("\n" + "=" * 105)
    print(f'Starting finite difference of "{type(function).__name__}" with dx = {dx}, and tol = {tol}')
    if isinstance(function, Network):
        sub = function.get_output_cone(tosig).get_input_cone(fromsig)
        if len(sub) == 0:
            raise RuntimeError(f"Could not find a network that use the provided input signals {fromsig} "
                               f"and produce the requested output signals {tosig}")
        inps = sub.sig_in if fromsig is None else _parse(fromsig)
        outps = sub.sig_out if tosig is None else _parse(tosig)
        if any(s.state is None for s in inps):
            function.get_output_cone(tosig=inps).response()
        function = sub
    else:
        inps = function.sig_in if fromsig is None else _parse(fromsig)
        outps = function.sig_out if tosig is None else _parse(tosig)
    print("Inputs:")
    print("\n".join(f"{i}\t{s.tag} = {s.state}" for i, s in enumerate(inps)) if verbose else
          ", ".join(s.tag for s in inps))
    print("")

    f0 = [None] * len(outps)
    df_an = [None] * len(outps)
    dx_an = [[None] * len(inps) for _ in outps]
    function.reset()
    function.response()
    print("Outputs:")
    print("\n".join(f"{i}\t{s.tag} = {s.state}" for i, s in enumerate(outps)) if verbose else
          ", ".join(s.tag for s in outps))
    for io, so in enumerate(outps):
        out = so.state
        if out is None:
            warnings.warn(f"Output {io} of {so.tag} is None")
            continue
        f0[io] = _copy(out)
        shape = tuple(out.shape) if hasattr(out, "shape") else ()
        if use_df is not None:
            d = use_df[io]
        else:
            d = np.random.rand(*shape) if random else np.ones(shape)
            if np.iscomplexobj(out) or (isinstance(out, torch.Tensor) and out.is_complex()):
                d = d + 1j * (np.random.rand(*shape) if random else np.ones(shape))
        if isinstance(out, torch.Tensor) and out.is_cuda and not isinstance(d, torch.Tensor):
            d = torch.as_tensor(np.asarray(d), device=out.device)
            d = d.reshape(()) if d.numel() == 1 and out.dim() == 0 else d
        df_an[io] = d
        so.sensitivity = d
        function.sensitivity()
        for ii, si in enumerate(inps):
            dx_an[io][ii] = _copy(si.sensitivity)
        function.reset()

    summary = {}
    for ii, si in enumerate(inps):
        print("_" * 51)
        print(f'Perturbing input {ii} "{si.tag}"...\n')
        x = si.state
        if isinstance(x, np.ndarray) and x.ndim > 0 and not x.flags.c_contiguous:
            x = np.ascontiguousarray(x)   # perturbed in place through a flat view
            si.state = x
        elif isinstance(x, torch.Tensor) and not x.is_contiguous():
            x = x.contiguous()
            si.state = x
        scalar = not (isinstance(x, torch.Tensor) or isinstance(x, np.ndarray)) or \
            (isinstance(x, np.ndarray) and x.ndim == 0)
        shape = () if scalar else tuple(x.shape)
        n = 1 if scalar else int(np.prod(shape))
        flat = None if scalar else x.reshape(-1)
        idx = range(n) if entries is None else [int(e) for e in np.atleast_1d(entries) if 0 <= int(e) < n]
        failed = tested = 0
        for e in idx:
            x0 = (x.item() if hasattr(x, "item") else x) if scalar else flat[e].item()
            if x0 == 0 and keep_zero_structure:
                continue
            sf = abs(x0) if (relative_dx and abs(x0) != 0) else 1.0
            parts = [(1.0, "")] + ([(1j, " (I)")] if isinstance(x0, complex) else [])
            for unit, label in parts:
                h = dx * unit * sf

                def respond(val):
                    if scalar:
                        si.state = val
                    else:
                        flat[e] = val
                        si.state = x
                    function.response()
                    return [_copy(so.state) for so in outps]

                fp = respond(x0 + h)
                fm = respond(x0 - h) if central else None
                for io, so in enumerate(outps):
                    if fp[io] is None or f0[io] is None:
                        warnings.warn(f"Output {io} of {so.tag} is None")
                        continue
                    ref = fm[io] if central else f0[io]
                    diff = (fp[io] - ref) / ((2.0 if central else 1.0) * h)
                    fd = _inner(diff, df_an[io])
                    an = _entry(dx_an[io][ii], e)
                    fd, an = (complex(fd).imag, complex(an).imag) if unit == 1j else (complex(fd).real,
                                                                                      complex(an).real)
                    if (abs(an) < tol) if unit == 1j else (abs(an) == 0):
                        err = abs(fd - an)
                    else:
                        err = abs(fd - an) / max(abs(fd), abs(an))
                    tested += 1
                    failed += int(err > tol)
                    if verbose or err > tol:
                        mi = np.unravel_index(e, shape) if shape else ()
                        print("δ%s/δ%s%s i = %s \tAn :% .3e \tFD : % .3e \tError: % .3e %s"
                              % (so.tag, si.tag, label, tuple(int(v) for v in mi), an, fd, err,
                                 "<--*" if err > tol else ""))
                    if test_fn is not None:
                        test_fn(x0, dx, an, fd)
                if scalar:
                    si.state = x0
                else:
                    flat[e] = x0
                    si.state = x
        print(f"-- Number of finite difference values beyond tolerance ({tol}) = {failed} / {tested}")
        summary[si.tag] = (failed, tested)
    function.response()   # leave the network at the unperturbed design
    print("_" * 51)
    print(f'\nFinished finite-difference check of "{type(function).__name__}"\n')
    print("=" * 105 + "\n")
    return summary


def minimize_oc(variables, objective, function=None, maxit=100, tolx=1e-4, tolf=1e-4, **kwargs):
    """pyMOTO's minimize_oc (pymoto/routines.py:300-316) with the device OC update."""
    from .optimizers import OC
    oc = OC(variables, objective, function, **kwargs)
    oc.optimize(maxiter=maxit, tolx=tolx, tolf=tolf)
    return oc


def minimize_mma(variables, responses, function=None, maxit=100, tolx=1e-4, tolf=1e-4, **kwargs):
    """pyMOTO's minimize_mma (pymoto/routines.py:320-338) with the device MMA update."""
    from .mma import MMA
    mma = MMA(variables, responses, function, **kwargs)
    mma.optimize(maxiter=maxit, tolx=tolx, tolf=tolf)
    return mma
