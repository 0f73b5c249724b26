"""Optimality-criteria optimizer on the device (pymoto/common/optimizers.py:337-437).

Same interface as pyMOTO's OC: OC(variables, response, function, move=0.1, xmin=0, xmax=1, ...).step() /
optimize().  The bisection on the Lagrange multiplier runs entirely on the device (pmg_oc_update), so a
design iteration needs no host copy of x or dg.  pyMOTO's own OC also works with the GPU modules when the
design Signal holds a numpy array.
"""
import torch

from ._lib import PMGError, call, stream
from .operators import Workspace
from .solvers import _from_device, _to_device


class OC:
    def __init__(self, variables, response, function, slice_network=False, move=0.1, xmin=0.0, xmax=1.0,
                 verbosity=2, l1init=0.0, l2init=100000.0, l1l2tol=1e-4, maxvol=None):
        self.variable = variables[0] if isinstance(variables, (list, tuple)) else variables
        self.response = response
        if function is None:
            from .core import Network
            function = Network.active[0]
        if slice_network:
            from .routines import slice_network as _slice
            function = _slice(function, [self.variable], [response])
        self.function = function
        self.move, self.xmin, self.xmax = float(move), float(xmin), float(xmax)
        self.verbosity = verbosity
        self.l1init, self.l2init, self.l1l2tol = float(l1init), float(l2init), float(l1l2tol)
        self.maxvol = maxvol
        self.iter = 0
        self.history = []

    def state_dict(self):
        """Iteration count, response history and the volume target (checkpoint)."""
        return {"iter": self.iter, "history": list(self.history), "maxvol": self.maxvol}

    def load_state_dict(self, sd):
        self.iter, self.history, self.maxvol = int(sd["iter"]), list(sd["history"]), sd["maxvol"]

    def _x(self):
        return _to_device(self.variable.state)

    def calculate_g(self):
        self.function.response()
        return float(self.response.state)

    def calculate_dg(self):
        self.function.reset()
        self.response.sensitivity = 1.0
        self.function.sensitivity()
        dg = self.variable.sensitivity
        self.function.reset()
        return dg

    def step(self):
        """One design iteration: response, sensitivities and the OC update of the design Signal."""
        x, kind = self._x()
        if self.maxvol is None:
            self.maxvol = float(x.sum().item()) / x.numel()
        self.function.response()
        ws = Workspace.get(x.device)
        if getattr(self, "_status", None) is None:
            self._status = torch.zeros(1, dtype=torch.int32).pin_memory()
            self._g_host = torch.zeros(1, dtype=torch.float64).pin_memory()
            self._g_event = torch.cuda.Event()
            self._status_event = torch.cuda.Event()
        if getattr(self, "_issued", False):
            # status of the previous update's bisection (a bounded wait that expired), copied to the host in
            # stream order after that update (complete by now when the response synchronised with the device)
            self._status_event.synchronize()
            if int(self._status[0]) != 0:
                raise PMGError("pmg_oc_update", 3, "the single-launch bisection's bounded wait expired")
        gs = self.response.state
        if isinstance(gs, torch.Tensor) and gs.is_cuda:
            # the response value is read once everything below is queued: no device idle time for it
            self._g_host.copy_(gs.reshape(1), non_blocking=True)
            self._g_event.record()
            g = None
        else:
            g = float(gs)
        dg = _to_device(self.calculate_dg(), device=x.device)[0]
        xnew = torch.empty_like(x)
        call("pmg_oc_update", x.numel(), x, dg, xnew, self.maxvol, self.move, self.xmin, self.xmax, self.l1init,
             self.l2init, self.l1l2tol, ws.oc, stream())
        call("pmg_oc_status_async", ws.oc, self._status, stream())
        self._status_event.record()
        self._issued = True
        self.variable.state = _from_device(xnew, kind)
        if g is None:
            self._g_event.synchronize()
            g = float(self._g_host[0])
        self.history.append(g)
        return xnew, g, dg

    def optimize(self, maxiter=100, tolx=1e-4, tolf=1e-4, evaluate_last=False):
        """pyMOTO's optimization loop (pymoto/common/optimizers.py:275-322): stop on the relative change of the
        response or of the design; the variables are left at the last evaluated design (at the new one, with
        its response computed, when evaluate_last)."""
        nom = type(self).__name__
        gcur = 0.0
        dxr = self.xmax - self.xmin
        last = None
        while self.iter < maxiter:
            xval, kind = self._x()       # the state tensor itself: step() replaces the state, not its values
            last = (xval, kind)
            xnew, g, _ = self.step()
            gprev, gcur = gcur, g
            rel_df = abs(gcur - gprev) / abs(gcur) if gcur != 0 else float("inf")
            if rel_df < tolf:
                if self.verbosity >= 1:
                    print(f"{nom} converged: Relative function change |Δf|/|f| ({rel_df}) below tolerance ({tolf})")
                self.variable.state = _from_device(xval, kind)
                break
            if self.verbosity >= 2:
                print("It. {0: 4d}, g0: {1:+.4e}".format(self.iter, g))
            rel_step = float((torch.linalg.vector_norm((xval - xnew) / dxr) /
                              torch.linalg.vector_norm(xval / dxr)).item())
            if rel_step < tolx:
                if self.verbosity >= 1:
                    print(f"{nom} converged: Relative stepsize |Δx|/|x| ({rel_step}) below tolerance ({tolx})")
                if evaluate_last:
                    self.function.response()
                else:
                    self.variable.state = _from_device(xval, kind)
                break
            self.iter += 1
        else:
            if last is not None:   # maxiter reached: the last new design was computed, not evaluated
                self.variable.state = _from_device(*last)
