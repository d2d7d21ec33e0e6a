"""FP64 oracle results of the full-size benchmark configurations, computed in
spawned worker processes while the GPU tests run.

The oracle's SuperLU factorizations of the 800 x 480 design-guide problem and
of the 1000 x 600 adjoint problem take tens of seconds each on one host core,
so the GPU tests that check against them submit the oracle work when pytest
has collected them (``start``) and read the results at the end (``result``).
The pool uses the ``spawn`` start method: a forked child of a process that has
touched the GPU can hang.
"""
from __future__ import annotations

import concurrent.futures as cf
import multiprocessing as mp
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_pool = None
_futures = {}


def _setup_paths():
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
        if p not in sys.path:
            sys.path.insert(0, p)
    import __graft_entry__
    __graft_entry__.load_package()


def job_design_guide():
    """Driven TM solve of the 800 x 480 design-guide problem (seed 2): Ez, Hx, Hy."""
    _setup_paths()
    import fdfd_oracle as O
    from fdfd_gb300 import workloads as W
    p = W.design_guide()
    g = O.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    return O.solve(g, p.eps, p.src, p.omega, O.TM, p.pml_m, p.pml_lnR)


def job_adjoint():
    """FP64 adjoint gradient of the 1000 x 600 adjoint problem: (J, grad, Ez)."""
    _setup_paths()
    import fdfd_oracle as O
    from fdfd_gb300 import workloads as W
    p = W.adjoint_problem()
    g = O.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    return O.adjoint_gradient(g, p.eps, p.src, p.omega, p.extra["mvec"], p.pml_m, p.pml_lnR)


def job_cavity():
    """The six TM eigenfrequencies of the 280 x 280 rod-lattice cavity nearest ωa/2πc = 0.38."""
    _setup_paths()
    import numpy as np
    import fdfd_oracle as O
    from fdfd_gb300 import workloads as W
    p, w0 = W.phc_cavity()
    g = O.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    w, _, _ = O.eigenfrequency(g, p.eps, w0, O.TM, 6, "LM", p.pml_m, p.pml_lnR,
                               v0=np.ones(p.Nx * p.Ny, dtype=complex))
    return w


JOBS = {"design_guide": job_design_guide, "adjoint": job_adjoint, "cavity": job_cavity}


def start(names):
    """Submit the named jobs (idempotent)."""
    global _pool
    names = [n for n in names if n not in _futures]
    if not names:
        return
    if _pool is None:
        # each worker runs SuperLU / ARPACK on one core; a few BLAS threads each
        for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
            os.environ.setdefault(k, "2")
        _pool = cf.ProcessPoolExecutor(max_workers=len(JOBS), mp_context=mp.get_context("spawn"))
    for n in names:
        _futures[n] = _pool.submit(JOBS[n])


def result(name, timeout=900):
    start([name])
    return _futures[name].result(timeout=timeout)


def shutdown():
    global _pool
    if _pool is not None:
        _pool.shutdown(wait=False, cancel_futures=True)
        _pool = None
