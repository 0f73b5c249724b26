"""Iteration log of scalar (and small vector) signals, from device values without a host synchronisation.

pyMOTO's ScalarToFile (pymoto/modules/io.py:351-419) formats every input signal's state each response and
appends one row to a text file (tab-separated, or comma-separated for .csv): the iteration number, then the
values in the given format, with a header row of the signal tags (vector entries as tag[i, j, ...]) written at
iteration 0.  The file is the same here.

What differs is where the time goes: in a GPU design loop the logged responses are 0-d CUDA tensors, and
formatting them where they are produced would stop the host until the device reaches that point every
iteration.  Here each response copies them into pinned host memory on the current stream and records an event;
a writer thread per module waits for the events, formats and appends the rows in order.  flush() waits for the
rows written so far.
"""
import atexit
import queue
import threading
from pathlib import Path

import numpy as np
import torch

from .core import Module, Signal


class ScalarToFile(Module):
    """pyMOTO's ScalarToFile: ScalarToFile(saveto, fmt=".10e", separator="\\t")(*signals)."""

    def __init__(self, saveto: str, fmt: str = ".10e", separator: str = "\t"):
        self.saveto = saveto
        Path(saveto).parent.mkdir(parents=True, exist_ok=True)
        self.iter = 0
        (3.14).__format__(fmt)   # reject an invalid format here, not in the writer thread
        self.format = fmt
        self.separator = "," if ".csv" in self.saveto else separator
        self._jobs = queue.Queue()
        self._error = None
        self._writer = threading.Thread(target=self._write_loop, daemon=True)
        self._writer.start()
        atexit.register(self.flush)

    def __call__(self, *args):
        if self.sig_in is None:
            raise NotImplementedError("Only for signals as inputs")
        staged, tags = [], ([] if self.iter == 0 else None)
        on_device = False
        for s in self.sig_in:
            if not isinstance(s, Signal):
                raise TypeError(f"Expected Signal, got {type(s)}")
            st = s.state
            if isinstance(st, torch.Tensor):
                if st.is_cuda:
                    h = torch.empty(st.shape, dtype=st.dtype, pin_memory=True)
                    h.copy_(st.detach(), non_blocking=True)
                    on_device = True
                else:
                    h = st.detach().clone()
                staged.append(h)
                shape = tuple(st.shape)
            else:
                a = np.array(st, copy=True)
                staged.append(a)
                shape = a.shape
            if tags is not None:
                if int(np.prod(shape)) > 1:
                    tags += [f"{s.tag}{list(ix)}" for ix in np.ndindex(*shape)]
                else:
                    tags.append(s.tag)
        event = None
        if on_device:   # the row is complete once the copies queued above have run
            event = torch.cuda.Event()
            event.record()
        self._raise_pending()
        self._jobs.put((self.iter, tags, staged, event))
        self.iter += 1

    def _row(self, it, staged):
        dat = [it.__format__("d")]
        for v in staged:
            a = v.numpy() if isinstance(v, torch.Tensor) else v
            if a.size > 1:
                dat += [x.__format__(self.format) for x in a.reshape(-1).tolist()]
            else:
                dat.append(a.reshape(-1)[0].item().__format__(self.format))
        return dat

    def _write_loop(self):
        while True:
            job = self._jobs.get()
            try:
                if job is None:
                    return
                it, tags, staged, event = job
                if event is not None:
                    event.synchronize()
                dat = self._row(it, staged)
                if tags is not None:
                    assert len(tags) == len(dat) - 1
                    with open(self.saveto, "w+") as f:
                        f.write(self.separator.join(["Iteration"] + tags))
                        f.write("\n")
                with open(self.saveto, "a+") as f:
                    f.write(self.separator.join(dat))
                    f.write("\n")
            except Exception as e:   # reported to the caller by the next __call__ or flush()
                self._error = e
            finally:
                self._jobs.task_done()

    def _raise_pending(self):
        if self._error is not None:
            e, self._error = self._error, None
            raise RuntimeError(f"ScalarToFile could not write {self.saveto}: {e}") from e

    def flush(self):
        """Wait until every row queued so far is in the file."""
        self._jobs.join()
        self._raise_pending()


class DesignLog:
    """One JSON line per design iteration (metrics of a run): record() takes the current values of the given
    signals (device scalars copied to pinned memory in stream order, like ScalarToFile), the solver's iteration
    counts, residual and fallback flag, the learned warm start's predictions, the optimizer's iteration and the
    host time since the previous record, plus any extra keyword values.  A background thread writes the lines."""

    def __init__(self, path, solver=None, optimizer=None, **signals):
        import time
        self._time = time.perf_counter
        self.path = path
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        open(path, "w").close()
        self.solver, self.optimizer, self.signals = solver, optimizer, signals
        self._t0 = self._time()
        self._jobs = queue.Queue()
        self._error = None
        threading.Thread(target=self._write_loop, daemon=True).start()
        atexit.register(self.flush)

    def _solver_fields(self):
        s = self.solver
        if s is None:
            return {}
        out = {k: getattr(s, k) for k in ("iterations", "last_residual", "inner_iterations", "fell_back")
               if hasattr(s, k)}
        ws = getattr(s, "warm_start", None)
        if ws is not None:
            out["learned_predictions"] = getattr(ws, "predictions", None)
        return {k: (v if isinstance(v, (bool, int, float, type(None))) else float(v)) for k, v in out.items()}

    def record(self, **extra):
        if self._error is not None:
            e, self._error = self._error, None
            raise RuntimeError(f"DesignLog could not write {self.path}: {e}") from e
        now = self._time()
        row = {"time_s": now - self._t0}
        self._t0 = now
        if self.optimizer is not None:
            row["iteration"] = getattr(self.optimizer, "iter", None)
        row.update(self._solver_fields())
        row.update(extra)
        staged, event = {}, None
        for name, sig in self.signals.items():
            st = getattr(sig, "state", sig)
            if isinstance(st, torch.Tensor) and st.is_cuda:
                h = torch.empty(st.shape, dtype=st.dtype, pin_memory=True)
                h.copy_(st.detach(), non_blocking=True)
                staged[name] = h
                event = event or torch.cuda.Event()
            else:
                staged[name] = st.detach().clone() if isinstance(st, torch.Tensor) else np.array(st, copy=True)
        if event is not None:
            event.record()
        self._jobs.put((row, staged, event))

    def _write_loop(self):
        import json
        while True:
            row, staged, event = self._jobs.get()
            try:
                if event is not None:
                    event.synchronize()
                for name, v in staged.items():
                    a = v.numpy() if isinstance(v, torch.Tensor) else v
                    row[name] = a.reshape(-1)[0].item() if a.size == 1 else a.reshape(-1).tolist()
                with open(self.path, "a") as f:
                    f.write(json.dumps(row) + "\n")
            except Exception as e:   # reported by the next record() or flush()
                self._error = e
            finally:
                self._jobs.task_done()

    def flush(self):
        self._jobs.join()
        if self._error is not None:
            e, self._error = self._error, None
            raise RuntimeError(f"DesignLog could not write {self.path}: {e}") from e
