"""Graph runtime the GPU modules plug into.

When pyMOTO is importable, its own Signal / Module / Network classes are used, so the modules of this
package drop into an existing pymoto Network and work with its optimizers (OC, MMA) and
finite_difference checker.  Otherwise the standalone runtime of `_graph` (same protocol) is used.
Set PYMOTO_GB300_STANDALONE=1 to force the standalone runtime.
"""
import os

_force_standalone = os.environ.get("PYMOTO_GB300_STANDALONE", "0") == "1"

try:
    if _force_standalone:
        raise ImportError
    from pymoto import Module, Network, Signal  # noqa: F401
    HOST_RUNTIME = "pymoto"
except Exception:  # pyMOTO (or its plotting dependency) is not available
    from ._graph import Module, Network, Signal  # noqa: F401
    HOST_RUNTIME = "standalone"
