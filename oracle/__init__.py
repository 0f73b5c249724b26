"""CPU oracle for the pymoto_gb300 hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy/scipy, the algorithm that pyMOTO (v2.0.1) runs for the
structured-grid compliance path: voxel numbering, element stiffness quadrature, CSR assembly with
Dirichlet rows, density filters, SIMP, geometric multigrid (prolongation, Galerkin product, damped
Jacobi, V-cycle, direct coarsest solve), block-PCG, the linear-dependency-aware wrapper, compliance,
the adjoint sensitivity contraction and the OC update.  Every function cites the pyMOTO file:line it
follows.

Only the test-suite, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it, and only as the checker or the timed CPU baseline.  The product path
(``pymoto_gb300``) never imports it and fails loudly when its CUDA library is missing.

Further restatements in their own modules: ``oracle.mma`` (MMA / subsolv, pymoto/common/mma.py) and
``oracle.overhang`` (the overhang filter's layer sweep, pymoto/modules/filter.py:381-713).

Parity pin: the oracle is checked against golden vectors written by running pyMOTO itself
(``tests/golden/make_golden.py``) and against pyMOTO's own known-answer tests (analytical bar in
tension, prolongation row sums, filter stencil placement).
"""
from .pymoto_oracle import *  # noqa: F401,F403
from .design_loop import (CachedHierarchy, ReferenceDesignLoop, StructuredCSR, cantilever_loads,  # noqa: F401,E402
                          fp64_cg_reference)
