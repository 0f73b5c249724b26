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

    def optimize(self, maxiter=100, tolx=1e-4, tolf=1e-4):
        gprev = 0.0
        while self.iter < maxiter:
            x, _ = self._x()
            xnew, g, _ = self.step()
            rel_df = abs(g - gprev) / abs(g) if g != 0 else 0.0
            gprev = g
            if self.verbosity >= 2:
                print(f"It. {self.iter}, g = {g:.6e}")
            if rel_df < tolf:
                self.variable.state = _from_device(x, _to_device(self.variable.state)[1])
                break
            dx = float(torch.linalg.vector_norm(x - xnew).item()) / max(float(torch.linalg.vector_norm(x).item()), 1e-300)
            self.iter += 1
            if dx < tolx:
                break
