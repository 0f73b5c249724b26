"""Standalone Signal / Module / Network runtime with pyMOTO's protocol.

Used when pyMOTO itself is not importable.  It follows the semantics of pymoto/core_objects.py:
  * Signal holds a state and a sensitivity; add_sensitivity deep-copies the first contribution and adds
    later ones in place (core_objects.py:107-135); reset zeroes or drops it (:137-165).
  * Module subclasses define __call__(*states) and _sensitivity(*dout); __init_subclass__ wraps __call__
    so that calling a module with Signals connects it, creates its output Signals and appends it to every
    active Network (:481-548).  Keyword-only arguments are rejected (:408-448).
  * Network runs response() in order and sensitivity() in reverse (:750-829); `with Network() as fn:`
    activates it; a default global network is always active (:998).  print_timing prints the host time of
    each module (:790-829); PYMOTO_GB300_NVTX=1 adds an NVTX range per module response and sensitivity.
"""
import copy
import inspect
import os
import sys
import time

# PYMOTO_GB300_NVTX=1: NVTX ranges around every module's response and sensitivity (for Nsight Systems)
_NVTX = os.environ.get("PYMOTO_GB300_NVTX", "0") == "1"
if _NVTX:
    import torch


def _as_list(x):
    if x is None:
        return []
    if isinstance(x, (list, tuple)):
        out = []
        for v in x:
            out.extend(_as_list(v)) if isinstance(v, (list, tuple)) else out.append(v)
        return out
    return [x]


class Signal:
    def __init__(self, tag: str = "", state=None, sensitivity=None, min=None, max=None):
        self.tag = tag
        self.state = state
        self.sensitivity = sensitivity
        self.min = min
        self.max = max
        self.keep_alloc = sensitivity is not None

    def add_sensitivity(self, ds):
        if ds is None:
            return self
        if self.sensitivity is None:
            clone = getattr(ds, "clone", None)
            # a device tensor is copied with clone() (deepcopy takes the slow Python-level path for the same copy)
            self.sensitivity = clone() if callable(clone) else copy.deepcopy(ds)
        elif hasattr(self.sensitivity, "add_sensitivity"):
            self.sensitivity.add_sensitivity(ds)
        else:
            self.sensitivity += ds
        return self

    def reset(self, keep_alloc: bool = None):
        if self.sensitivity is None:
            return self
        keep = self.keep_alloc if keep_alloc is None else keep_alloc
        if keep:
            try:
                self.sensitivity[...] = 0
            except TypeError:
                self.sensitivity *= 0
        else:
            self.sensitivity = None
        return self

    def __repr__(self):
        return f"Signal '{self.tag}'"


def _is_signal(s):
    return isinstance(s, Signal) or (hasattr(s, "state") and hasattr(s, "add_sensitivity"))


def _check_signature(fn, n_args=None):
    lo, hi = 0, 0
    for p in inspect.signature(fn).parameters.values():
        if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD):
            if p.default is p.empty:
                lo += 1
            if hi is not None:
                hi += 1
        elif p.kind == p.VAR_POSITIONAL:
            hi = None
        else:
            raise SyntaxError(f"{fn.__qualname__} may not have keyword-only arguments ({p})")
    if n_args is not None:
        if n_args < lo or (hi is not None and n_args > hi):
            raise TypeError(f"{fn.__qualname__} takes {lo}..{hi} arguments, {n_args} given")
    return lo, hi


class Module:
    sig_in = None
    sig_out = None

    def __init_subclass__(cls, **kwargs):
        super().__init_subclass__(**kwargs)
        fwd = cls.__dict__.get("__call__")
        if fwd is None or getattr(fwd, "_pmg_wrapped", False):
            return
        _check_signature(fwd)
        cls._orig_call = fwd
        cls._response = cls._wrap(fwd, create=False)
        cls.__call__ = cls._wrap(fwd, create=True)

    @classmethod
    def _wrap(cls, fn, create):
        def wrapped(self, *args):
            states = [a.state if _is_signal(a) else a for a in args]
            constant = len(args) > 0 and not any(_is_signal(a) for a in args)
            if create and not constant:
                self.sig_in = list(args)
            out = fn(self, *states)
            if constant:
                return out
            outs = _as_list(out) if isinstance(out, (list, tuple)) or out is None else [out]
            if create:
                if self.sig_out is None:
                    self.sig_out = [Signal(f"{type(self).__name__}_output{i}") for i in range(len(outs))]
                _check_signature(self._sensitivity, len(self.sig_out))
                for n in Network.active:
                    if self in n.mods:
                        raise RuntimeError("Module already in network, cannot add twice.")
                    n.append(self)
            if len(outs) != len(self.sig_out):
                raise TypeError("number of responses does not match the number of output signals")
            for s, v in zip(self.sig_out, outs):
                s.state = v
            if len(self.sig_out) == 0:
                return None
            return self.sig_out[0] if len(self.sig_out) == 1 else tuple(self.sig_out)

        wrapped._pmg_wrapped = True
        return wrapped

    @property
    def n_in(self):
        return None if self.sig_in is None else len(self.sig_in)

    @property
    def n_out(self):
        return None if self.sig_out is None else len(self.sig_out)

    def response(self):
        try:
            self._response(*self.sig_in)
            return self
        except Exception as e:
            raise type(e)(f"{e}\n\t| raised in response() of {type(self).__name__}").with_traceback(sys.exc_info()[2])

    def sensitivity(self):
        try:
            douts = [s.sensitivity if _is_signal(s) else None for s in (self.sig_out or [])]
            if self.n_out and all(d is None for d in douts):
                return self
            dins = self._sensitivity(*douts)
            dins = _as_list(dins) if isinstance(dins, (list, tuple)) else [dins]
            if len(dins) != self.n_in:
                raise TypeError("number of sensitivities does not match the number of input signals")
            for s, d in zip(self.sig_in, dins):
                if _is_signal(s):
                    s.add_sensitivity(d)
            return self
        except Exception as e:
            raise type(e)(f"{e}\n\t| raised in sensitivity() of {type(self).__name__}").with_traceback(
                sys.exc_info()[2])

    def reset(self):
        for s in (self.sig_out or []) + (self.sig_in or []):
            if _is_signal(s):
                s.reset()
        self._reset()
        return self

    def get_input_states(self, as_list=False):
        st = [s.state if _is_signal(s) else s for s in self.sig_in]
        return st[0] if (len(st) == 1 and not as_list) else st

    def get_output_states(self, as_list=False):
        st = [s.state for s in self.sig_out]
        return st[0] if (len(st) == 1 and not as_list) else st

    def _sensitivity(self, *args):
        return [None for _ in self.sig_in]

    def _reset(self):
        pass


class Network(Module):
    active = []

    def __init__(self, *mods, print_timing=False):
        self.mods = []
        self.print_timing = print_timing
        self.append(*mods)

    def __enter__(self):
        if self in Network.active:
            raise ValueError("Network is already activated")
        Network.active.append(self)
        return self

    def __exit__(self, *exc):
        Network.active.remove(self)

    def append(self, *mods):
        ml = _as_list(list(mods))
        for m in ml:
            if not isinstance(m, Module):
                raise TypeError(f"not a module: {type(m).__name__}")
        self.mods.extend(ml)
        if ml:
            return ml[-1].sig_out[0] if len(ml[-1].sig_out) == 1 else ml[-1].sig_out

    def _run(self, fn, label):
        if _NVTX:   # a named range per module response / sensitivity for Nsight timelines
            torch.cuda.nvtx.range_push(label.strip("- "))
            try:
                self._timed(fn, label)
            finally:
                torch.cuda.nvtx.range_pop()
            return
        self._timed(fn, label)

    def _timed(self, fn, label):
        if self.print_timing is False:
            fn()
            return
        t0 = time.time()
        fn()
        dt = time.time() - t0
        tmin = 0.0 if isinstance(self.print_timing, bool) else self.print_timing
        if dt > tmin:
            print(f"{label} took {dt} s")

    def response(self):
        for m in self.mods:
            self._run(m.response, f'-- Response of "{type(m).__name__}"')

    def sensitivity(self):
        for m in reversed(self.mods):
            self._run(m.sensitivity, f'-- Sensitivity of "{type(m).__name__}"')

    def reset(self):
        for m in reversed(self.mods):
            m.reset()

    def __len__(self):
        return len(self.mods)

    def __iter__(self):
        return iter(self.mods)

    def __getitem__(self, i):
        return self.mods[i]

    def __call__(self, *args):
        raise RuntimeError("Cannot re-connect signals in existing network")

    @staticmethod
    def _signal_set(sigs):
        if sigs is None:
            return set()
        return {s for s in (_as_list(sigs) if isinstance(sigs, (list, tuple)) else [sigs]) if _is_signal(s)}

    def _stubs(self):
        all_in, all_out = set(), set()
        for m in self.mods:
            all_in |= self._signal_set(m.sig_in)
            all_out |= self._signal_set(m.sig_out)
        return all_in, all_out

    @property
    def sig_in(self):
        """Input signals no module of the network produces (core_objects.py:895-902)."""
        all_in, all_out = self._stubs()
        return list(all_in - all_out)

    @sig_in.setter
    def sig_in(self, v):
        raise RuntimeError("Cannot re-connect signals in existing network")

    @property
    def sig_out(self):
        """Output signals no module of the network uses (core_objects.py:904-911)."""
        all_in, all_out = self._stubs()
        return list(all_out - all_in)

    @sig_out.setter
    def sig_out(self, v):
        raise RuntimeError("Cannot re-connect signals in existing network")

    def get_input_cone(self, fromsig=None, frommod=None):
        """The modules that depend on `fromsig` / `frommod`, in network order (core_objects.py:913-928)."""
        touched = self._signal_set(fromsig)
        frommod = set(_as_list(frommod) if isinstance(frommod, (list, tuple)) else ([] if frommod is None else
                                                                                   [frommod]))
        if not touched and not frommod:
            return self
        cone = Network()
        for m in self.mods:
            if m in frommod or self._signal_set(m.sig_in) & touched:
                touched |= self._signal_set(m.sig_out)
                cone.mods.append(m)
        return cone

    def get_output_cone(self, tosig=None, tomod=None):
        """The modules `tosig` / `tomod` depend on, in network order (core_objects.py:930-945)."""
        dependent = self._signal_set(tosig)
        tomod = set(_as_list(tomod) if isinstance(tomod, (list, tuple)) else ([] if tomod is None else [tomod]))
        if not dependent and not tomod:
            return self
        cone = []
        for m in reversed(self.mods):
            if m in tomod or self._signal_set(m.sig_out) & dependent:
                dependent |= self._signal_set(m.sig_in)
                cone.append(m)
        out = Network()
        out.mods = list(reversed(cone))
        return out


Network.active.append(Network())
