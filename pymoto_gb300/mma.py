"""Method of Moving Asymptotes with the update on the device (pymoto/common/mma.py, pymoto/common/optimizers.py).

Same interface as pyMOTO's MMA: MMA(variables, responses, function, slice_network=False, move=0.1, xmin=0.0,
xmax=1.0, verbosity=2, mmaversion="MMA2007", **kwargs).step(x, g, dg) / optimize(maxiter, tolx, tolf), with
pyMOTO's options (a0, epsimin, cCoef, albefa, asyinit, asyincr, asydecr, asybound, gcmma_maxit, a, c) and
versions MMA1987, MMA2007 and GCMMA, plus exact=True for numpy's rounding of every element-wise value.  The asymptote adaptation, the separable approximation and the whole
interior-point subproblem solve run in one cooperative CUDA launch (pmg_mma_update); design, sensitivities,
offsets and asymptotes stay on the device.  The responses are read on the host only where pyMOTO reads them
(the convergence test of optimize, the GCMMA acceptance test).
"""
import ctypes
import math

import numpy as np
import torch

from ._lib import PMGError, call, stream
from .solvers import _from_device, _to_device

MAX_M = 4
_VERSIONS = {"1987": 0, "2007": 1, "gcmma": 2}


class _Params(ctypes.Structure):
    """pmg_mma_params of include/pymoto_gb300.h."""
    _fields_ = [("version", ctypes.c_int), ("m", ctypes.c_int), ("adapt", ctypes.c_int), ("maxit", ctypes.c_int),
                ("exact", ctypes.c_int), ("reserved", ctypes.c_int),
                ("a0", ctypes.c_double), ("albefa", ctypes.c_double), ("asyincr", ctypes.c_double),
                ("asydecr", ctypes.c_double), ("offmin", ctypes.c_double), ("offmax", ctypes.c_double),
                ("epsimin", ctypes.c_double), ("rho", ctypes.c_double * (MAX_M + 1)),
                ("a", ctypes.c_double * MAX_M), ("c", ctypes.c_double * MAX_M), ("d", ctypes.c_double * MAX_M)]


def _version_code(name):
    low = name.lower()
    for key, code in _VERSIONS.items():
        if key in low:
            return code
    raise ValueError('Only "MMA1987", "MMA2007", or "GCMMA" are valid options')


class MMAUpdate:
    """The device state of an MMA run (offsets, previous designs, asymptotes) and its update
    x, g, dg -> xnew (mma.py:96-234).  Used by MMA; usable alone with device tensors.

    exact=True divides wherever pyMOTO divides, so every element-wise value rounds as numpy's; the default
    (False) inverts each denominator once, about 3x fewer FP64 divisions, with the same subproblem solution to
    its tolerance."""

    def __init__(self, n, m_resp, xmin, xmax, move=0.1, mmaversion="MMA2007", a0=1.0, epsimin=1e-10, cCoef=1e3,
                 albefa=0.1, asyinit=0.5, asyincr=1.2, asydecr=0.7, asybound=10.0, a=None, c=None, device=None,
                 maxit=400, exact=False):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.n = int(n)
        self.m = max(1, int(m_resp) - 1)
        if self.m > MAX_M:
            raise NotImplementedError(f"the device MMA update supports at most {MAX_M} constraints, got {self.m}")
        self.version = _version_code(mmaversion)
        full = lambda v: torch.full((self.n,), float(v), dtype=torch.float64, device=self.device)  # noqa: E731
        self.xmin = xmin if isinstance(xmin, torch.Tensor) else full(xmin)
        self.xmax = xmax if isinstance(xmax, torch.Tensor) else full(xmax)
        self.move = move if isinstance(move, torch.Tensor) else full(move)
        self.dx = self.xmax - self.xmin
        self.a0, self.epsimin, self.albefa = float(a0), float(epsimin), float(albefa)
        self.asyincr, self.asydecr, self.asybound = float(asyincr), float(asydecr), float(asybound)
        self.maxit = int(maxit)
        self.exact = bool(exact)
        self.offset = full(asyinit)
        self.xold1 = self.xold2 = None
        self.low = self.upp = None
        self.a = np.zeros(self.m) if a is None else np.asarray(a, dtype=float)
        if len(self.a) != self.m:
            raise RuntimeError(f"Length of the a vector ({len(self.a)}) should be equal to # constraints ({self.m}).")
        self.c = np.full(self.m, cCoef, dtype=float) if c is None else np.asarray(c, dtype=float)
        if len(self.c) != self.m:
            raise RuntimeError(f"Length of the c vector ({len(self.c)}) should be equal to # constraints ({self.m}).")
        self.d = np.ones(self.m)
        self.scratch = torch.empty(call("pmg_mma_scratch_bytes", self.n, self.m), dtype=torch.uint8,
                                   device=self.device)
        self.info = torch.zeros(self.m + 6, dtype=torch.float64, device=self.device)
        self._info_host = torch.zeros(self.m + 6, dtype=torch.float64).pin_memory()
        self._info_event = torch.cuda.Event()
        self._pending = False
        self._unconstrained = False
        self._zero_row = None
        self._minus_one = torch.tensor([-1.0], dtype=torch.float64, device=self.device)

    def state_dict(self):
        """Asymptote offsets and the two previous designs (checkpoint)."""
        return {"offset": self.offset, "xold1": self.xold1, "xold2": self.xold2}

    def load_state_dict(self, sd):
        self._check()
        self.offset.copy_(sd["offset"].to(self.offset.device))
        self.xold1 = None if sd["xold1"] is None else sd["xold1"].to(self.device)
        self.xold2 = None if sd["xold2"] is None else sd["xold2"].to(self.device)

    def adapt_ready(self):
        return self.xold1 is not None and self.xold2 is not None

    def mmasub(self, xval, g, dg, rho=1e-5, adapt=False):
        """New design from the responses g (m_resp,) and sensitivities dg (m_resp, n), device FP64 tensors; the
        offsets adapt first when `adapt` (mma.py:110-126, done once per outer MMA step)."""
        self._check()
        g = g.reshape(-1).to(device=self.device, dtype=torch.float64)
        dg = dg.reshape(-1, self.n).to(device=self.device, dtype=torch.float64)
        self._unconstrained = g.numel() == 1
        if self._unconstrained:   # dummy constraint -1 with zero sensitivities (mma.py:172-175)
            if self._zero_row is None:
                self._zero_row = torch.zeros((1, self.n), dtype=torch.float64, device=self.device)
            g = torch.cat([g, self._minus_one])
            dg = torch.cat([dg, self._zero_row])
        if g.numel() != self.m + 1:
            raise ValueError(f"{g.numel()} responses for {self.m} constraints")
        g, dg = g.contiguous(), dg.contiguous()
        p = _Params()
        p.version, p.m, p.adapt, p.maxit = self.version, self.m, int(bool(adapt) and self.adapt_ready()), self.maxit
        p.exact = int(self.exact)
        p.a0, p.albefa, p.asyincr, p.asydecr = self.a0, self.albefa, self.asyincr, self.asydecr
        p.offmin, p.offmax = 1 / (self.asybound ** 2), self.asybound
        p.epsimin = self.epsimin * math.sqrt(self.m + self.n)
        r = np.atleast_1d(np.asarray(rho, dtype=float))
        if r.size == 1:   # one value broadcasts over all rows, as numpy's rho[:, None] does
            r = np.full(self.m + 1, r[0])
        for i in range(min(r.size, MAX_M + 1)):
            p.rho[i] = r[i]
        for i in range(self.m):
            p.a[i], p.c[i], p.d[i] = self.a[i], self.c[i], self.d[i]
        xval = xval.reshape(-1).to(device=self.device, dtype=torch.float64).contiguous()
        self.low = torch.empty_like(xval)
        self.upp = torch.empty_like(xval)
        xnew = torch.empty_like(xval)
        call("pmg_mma_update", self.n, ctypes.addressof(p), xval, self.xold1, self.xold2, self.xmin, self.xmax,
             self.move, g, dg, self.offset, self.low, self.upp, xnew, self.info, self.scratch, stream())
        self._info_host.copy_(self.info, non_blocking=True)
        self._info_event.record()
        self._pending = True
        return xnew

    def step(self, xval, g, dg, rho=1e-5):
        """One MMA step (adaptation + mmasub), then xold2, xold1 = xold1, xval (mma.py:96-168)."""
        xnew = self.mmasub(xval, g, dg, rho, adapt=True)
        self.shift_history(xval)
        return xnew

    def shift_history(self, xval):
        self.xold2, self.xold1 = self.xold1, xval.reshape(-1).to(self.device, torch.float64).clone()

    def _check(self):
        """Status of the previous update (read once its copy to the host has completed)."""
        if self._pending:
            self._info_event.synchronize()
            self._pending = False
            st = int(self._info_host[self.m + 2])
            if st != 0:
                why = "a bounded wait expired" if st == 1 else "the Newton system of the subproblem is singular"
                raise PMGError("pmg_mma_update", 3 if st == 1 else 2, why)

    def _info(self):
        self._check()
        return self._info_host.numpy()

    @property
    def gest(self):
        v = self._info()[:self.m + 1].copy()
        return v[[0]] if self._unconstrained else v

    @property
    def dk(self):
        return float(self._info()[self.m + 1])

    @property
    def stats(self):
        i = self._info()
        return {"outer": int(i[self.m + 3]), "newton": int(i[self.m + 4]), "trials": int(i[self.m + 5])}


class MMA:
    """pyMOTO's MMA optimizer (pymoto/common/mma.py:5-168 with Optimizer, pymoto/common/optimizers.py:9-336)."""

    def __init__(self, variables, responses, function=None, slice_network=False, move=0.1, xmin=0.0, xmax=1.0,
                 verbosity=2, mmaversion="MMA2007", **kwargs):
        self.variables = list(variables) if isinstance(variables, (list, tuple)) else [variables]
        self.responses = list(responses) if isinstance(responses, (list, tuple)) else [responses]
        if function is None:
            from .core import Network
            function = Network.active[0]
        if slice_network:
            from .routines import slice_network as _slice
            function = _slice(function, self.variables, self.responses)
        self.function = function
        self.verbosity = verbosity
        self.response_is_uptodate = not any(s.state is None for s in self.responses)
        devs = [_to_device(s.state) for s in self.variables]
        self._kinds = [k for _, k in devs]
        sizes = [t.numel() for t, _ in devs]
        self._cumlens = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
        self.n = int(self._cumlens[-1])
        self.device = devs[0][0].device
        if xmin is None and all(hasattr(s, "min") for s in self.variables):
            xmin = [s.min for s in self.variables]
        if xmax is None and all(hasattr(s, "max") for s in self.variables):
            xmax = [s.max for s in self.variables]
        self.xmin = self._parse_bound(xmin, "xmin")
        self.xmax = self._parse_bound(xmax, "xmax")
        self.move = self._parse_bound(move, "move")
        self.mmaversion = mmaversion
        self.gcmma_maxit = kwargs.get("gcmma_maxit", 20)
        opts = {k: kwargs[k] for k in ("a0", "epsimin", "cCoef", "albefa", "asyinit", "asyincr", "asydecr",
                                       "asybound", "a", "c", "exact") if k in kwargs}
        self.core = MMAUpdate(self.n, len(self.responses), self.xmin, self.xmax, self.move, mmaversion,
                              device=self.device, **opts)
        self.m = self.core.m
        self.dx = self.core.dx
        self.iter = 0
        self.rho = None
        self.gest = None
        self.dk = None

    def state_dict(self):
        """Iteration count, the update's state and GCMMA's rho (checkpoint)."""
        rho = self.rho.tolist() if isinstance(self.rho, np.ndarray) else self.rho
        return {"iter": self.iter, "core": self.core.state_dict(), "rho": rho}

    def load_state_dict(self, sd):
        self.iter = int(sd["iter"])
        self.core.load_state_dict(sd["core"])
        # the design signals are restored beside this state: responses computed before the restore are stale
        self.response_is_uptodate = False
        self.rho = np.asarray(sd["rho"], dtype=float) if isinstance(sd["rho"], list) else sd["rho"]

    # --- pyMOTO Optimizer protocol ---------------------------------------------------------------------
    def _parse_bound(self, xbnd, which="bounds"):
        """Per-variable bound vector on the device (optimizers.py:95-121)."""
        if isinstance(xbnd, torch.Tensor):
            v = xbnd.to(device=self.device, dtype=torch.float64).reshape(-1)
            return v.expand(self.n).contiguous() if v.numel() == 1 else v.contiguous()
        try:
            nb = np.size(xbnd)
        except ValueError:
            nb = len(xbnd)
        if nb == 1:
            b = np.full(self.n, float(np.asarray(xbnd).ravel()[0]))
        elif nb == len(self.variables):
            b = np.zeros(self.n)
            for i in range(nb):
                b[self._cumlens[i]:self._cumlens[i + 1]] = xbnd[i]
        elif nb == self.n:
            b = np.asarray(xbnd, dtype=float).ravel()
        else:
            raise RuntimeError(f"Size of {which} ({nb}) should be either: scalar, the number of variable signals "
                               f"({len(self.variables)}) or the number of design variables ({self.n})")
        return torch.as_tensor(b, dtype=torch.float64, device=self.device).contiguous()

    @property
    def x(self):
        """The design vector (device FP64)."""
        parts = [_to_device(s.state, device=self.device)[0].reshape(-1) for s in self.variables]
        return parts[0] if len(parts) == 1 else torch.cat(parts)

    @x.setter
    def x(self, v):
        for i, s in enumerate(self.variables):
            lo, hi = self._cumlens[i], self._cumlens[i + 1]
            part = v[lo:hi]
            cur = s.state
            if isinstance(cur, torch.Tensor) and cur.is_cuda and cur.numel() == part.numel() and \
                    cur.data_ptr() == part.data_ptr():
                continue
            val = _from_device(part.contiguous(), self._kinds[i])
            s.state = val[0] if hi - lo == 1 else val
            self.response_is_uptodate = False

    def calculate_g(self):
        """Responses as a device FP64 vector (optimizers.py:144-156)."""
        if not self.response_is_uptodate:
            self.function.response()
            self.response_is_uptodate = True
        vals = []
        for s in self.responses:
            st = s.state
            if st is None:
                raise ValueError("Response is `None` and may not yet been calculated.")
            if isinstance(st, torch.Tensor):
                if st.is_complex():
                    raise TypeError("Responses for optimization must be real-valued.")
                if st.numel() > 1:
                    raise TypeError("Responses for optimziation must be scalar.")
                vals.append(st.reshape(()).to(device=self.device, dtype=torch.float64))
            else:
                if np.iscomplexobj(st):
                    raise TypeError("Responses for optimization must be real-valued.")
                if np.asarray(st).size > 1:
                    raise TypeError("Responses for optimziation must be scalar.")
                vals.append(torch.tensor(float(np.asarray(st).ravel()[0]), dtype=torch.float64, device=self.device))
        return torch.stack(vals)

    def calculate_dg(self):
        """Jacobian (m_resp, n) on the device by one back-propagation per response (optimizers.py:158-172)."""
        rows = []
        self.function.reset()
        for s_out in self.responses:
            s_out.sensitivity = 1.0
            self.function.sensitivity()
            parts = []
            for v in self.variables:
                sv = v.sensitivity
                if sv is None:
                    parts.append(torch.zeros(_to_device(v.state, device=self.device)[0].numel(), dtype=torch.float64,
                                             device=self.device))
                else:
                    parts.append(_to_device(sv, device=self.device)[0].reshape(-1))
            rows.append(parts[0] if len(parts) == 1 else torch.cat(parts))
            self.function.reset()
        return torch.stack(rows)

    # --- MMA ------------------------------------------------------------------------------------------
    def step(self, x=None, g=None, dg=None):
        """One (GC)MMA step; returns (xnew, g, dg) as device tensors (mma.py:96-168)."""
        if x is None:
            x = self.x
        else:
            x = _to_device(x, device=self.device)[0].reshape(-1)
            self.x = x
        is_gcmma = "gcmma" in self.mmaversion.lower()
        max_it = self.gcmma_maxit if is_gcmma else 1
        xnew = None
        gk = None
        for it in range(max_it):
            if it > 0:
                self.x = xnew
            if g is None or it > 0:
                g = self.calculate_g()
            else:
                g = _to_device(g, device=self.device)[0].reshape(-1)
            if it == 0:
                gk = g
            if dg is None:
                dg = self.calculate_dg()
            else:
                dg = _to_device(dg, device=self.device)[0].reshape(len(self.responses), self.n)
            if not is_gcmma:
                self.rho = 1e-5
            elif it > 0:
                gh = g.cpu().numpy()
                gest = self.core.gest
                if np.all(gest >= gh):
                    if self.verbosity >= 3:
                        print(f"  || GCMMA converged in {it} inner iterations")
                    break
                delta = (gh - gest) / self.core.dk
                upd = np.minimum(1.1 * (self.rho + delta), 10 * self.rho)
                self.rho[delta > 0] = upd[delta > 0]
                if self.verbosity >= 3:
                    print(f"  || GCMMA It. {it}, g = {gh}, gest = {gest}, rho={self.rho}")
            else:
                self.rho = (0.1 / self.n * torch.sum(self.dx * torch.abs(dg), dim=1)).cpu().numpy()
            xnew = self.core.mmasub(x, gk, dg, rho=self.rho, adapt=(it == 0))
        self.core.shift_history(x)
        return xnew, g, dg

    @property
    def low(self):
        return self.core.low

    @property
    def upp(self):
        return self.core.upp

    @property
    def offset(self):
        return self.core.offset

    def optimize(self, maxiter=100, tolx=1e-4, tolf=1e-4, evaluate_last=False):
        """pyMOTO's optimization loop (optimizers.py:275-322)."""
        nom = type(self).__name__
        xval = self.x
        gcur = np.zeros(1)
        while self.iter < maxiter:
            xnew, g, dg = self.step(x=xval)
            gh = g.cpu().numpy()
            gprev, gcur = gcur, gh
            rel_df = np.linalg.norm(gcur - gprev) / np.linalg.norm(gcur)
            if rel_df < tolf:
                if self.verbosity >= 1:
                    print(f"{nom} converged: Relative function change |Δf|/|f| ({rel_df}) below tolerance ({tolf})")
                break
            if self.verbosity >= 2:
                msgs = ["g{0:d}({1:s}): {2:+.4e}".format(i, getattr(s, "tag", str(i)), gh[i])
                        for i, s in enumerate(self.responses)]
                feas = ("[f] " if max(gh[1:]) <= 0 else "[ ] ") if len(self.responses) > 1 else ""
                print("It. {0: 4d}, {1:s}{2}".format(self.iter, feas, ", ".join(msgs)))
            rel_step = float((torch.linalg.vector_norm((xval - xnew) / self.dx) /
                              torch.linalg.vector_norm(xval / self.dx)).item())
            if rel_step < tolx:
                if self.verbosity >= 1:
                    print(f"{nom} converged: Relative stepsize |Δx|/|x| ({rel_step}) below tolerance ({tolx})")
                if evaluate_last:
                    self.x = xnew
                    self.calculate_g()
                break
            xval = xnew
            self.iter += 1
