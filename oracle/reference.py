"""Adapter that runs the reference's own RHF-CCSD code (CrawfordGroup/pycc) on a synthetic
Hamiltonian -- TEST INFRASTRUCTURE ONLY.

The reference is pure Python.  Its integral source needs psi4 and qcelemental, which are
not installed, but the CCSD arithmetic never touches them: ``import_reference`` puts inert
stand-ins for both modules into ``sys.modules`` (only module-level physical constants are
read from them, e.g. ``pycc/ccresponse.py:27-28``, ``pycc/properties.py:31-34``) and imports
``pycc`` from a given tree.  ``make_ref_ccwfn`` assembles a ``pycc.ccwfn.CCwfn`` with
``CCwfn.__new__`` plus the attributes ``CCwfn.__init__`` would set
(``pycc/ccwfn.py:76-213``, ``pycc/wavefunction.py:293-332``, ``pycc/device.py:116-154``),
so ``residuals`` / ``solve_cc`` / ``cc_energy`` / ``helper_diis`` and the (T), Lambda and
density drivers run unmodified.

Users: ``tests/golden/make_golden.py`` (the fixtures) and the CPU legs of ``bench.py``,
which time the reference's own iteration on the host cores.  Nothing in the engine imports
this module.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np


def import_reference(path):
    """Import the reference package ``pycc`` from the directory ``path`` (a source tree or a
    ``pip install --target`` directory) with psi4 / qcelemental stand-ins.

    Raises ImportError when ``path`` holds no ``pycc`` package or its dependencies
    (numpy, opt_einsum) are missing."""
    if not path or not os.path.isdir(os.path.join(path, "pycc")):
        raise ImportError("no reference package 'pycc' under %r" % (path,))
    sys.dont_write_bytecode = True
    for name in ("psi4", "qcelemental"):
        if name not in sys.modules:
            mod = types.ModuleType(name)
            consts = types.SimpleNamespace(get=lambda *a, **k: 1.0,
                                           conversion_factor=lambda *a, **k: 1.0)
            mod.constants = consts
            mod.core = types.SimpleNamespace()
            sys.modules[name] = mod
    if path not in sys.path:
        sys.path.insert(0, path)
    import pycc  # noqa: F401
    return pycc


class _H:
    """Stand-in for ``pycc.hamiltonian.Hamiltonian``: the four arrays the CCSD path reads."""


def make_ref_ccwfn(pycc, F, ERI, L, no, nv, model="CCSD"):
    """A reference ``CCwfn`` on the host arrays (F, ERI, L) in the reference's layout, at its
    MP2 guess (``pycc/ccwfn.py:195-211``), with the CPU double-precision backend."""
    from pycc.ccwfn import CCwfn
    from pycc.device import DeviceManager
    w = CCwfn.__new__(CCwfn)
    w.model = model
    w.method = model
    w.orbital_basis = "spatial"
    w.local = None
    w.need_singles = ['CCSD', 'CCSD(T)', 'CC2', 'CC3']
    w.make_t3_density = False
    w.store_triples = False
    w.real_time = False
    w.field = False
    w.nfzc = 0
    w.no, w.nv, w.nmo = no, nv, no + nv
    w.o = slice(0, no)
    w.v = slice(no, no + nv)
    H = _H()
    H.F = F
    H.eps = np.diag(F).copy()
    H.ERI = ERI
    H.L = L
    w.H = H
    w.eref = 0.0
    mgr = DeviceManager('CPU', 'DP')
    w.device_manager = mgr
    w.contract = mgr.contract
    w.precision = 'DP'
    w.device = 'CPU'
    w.device0 = None
    w.device1 = None
    w.e_conv = 1e-7
    w.r_conv = 1e-7
    w.maxiter = 100
    o, v = w.o, w.v
    eps_o, eps_v = H.eps[o], H.eps[v]
    w.Dijab = (eps_o.reshape(-1, 1, 1, 1) + eps_o.reshape(-1, 1, 1)
               - eps_v.reshape(-1, 1) - eps_v)
    w.Dia = eps_o.reshape(-1, 1) - eps_v
    w.t1 = np.zeros((no, nv))
    w.t2 = ERI[o, o, v, v].copy() / w.Dijab
    return w


class _Stop(Exception):
    pass


def time_solve_iterations(w, warmup, steps, budget_s=None, clock=None):
    """Time the reference's own ``solve_cc`` iterations (``pycc/ccwfn.py:268-319``: residual,
    Jacobi update and norm, energy, convergence test, DIIS) without changing its code.

    ``solve_cc`` runs with ``e_conv = r_conv = 0`` (so it never stops early) and
    ``maxiter = warmup + steps``; a wrapper around the instance's ``residuals`` records when
    each iteration starts.  Iteration k's time is the gap between the starts of k and k+1
    (the last one ends when ``solve_cc`` returns).  When ``budget_s`` is given, the wrapper
    stops the loop at the first iteration boundary after the timed iterations have used
    that many seconds, so only whole iterations are counted.

    Returns (per-iteration seconds of the timed iterations, warm-up iterations run)."""
    import contextlib
    import io
    import time
    clock = clock or time.perf_counter
    starts = []
    orig = w.residuals

    def timed(*a, **k):
        now = clock()
        starts.append(now)
        if budget_s is not None and len(starts) > warmup + 1 and \
                now - starts[warmup] > budget_s:
            raise _Stop()
        return orig(*a, **k)

    w.residuals = timed
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            try:
                w.solve_cc(0.0, 0.0, warmup + steps, 8, 1)
                starts.append(clock())
            except (_Stop, np.linalg.LinAlgError):
                # a budget stop, or a DIIS system that became singular long after
                # convergence: the iterations before it are whole
                pass
    finally:
        del w.residuals
    gaps = [b - a for a, b in zip(starts[:-1], starts[1:])]
    return gaps[warmup:], min(warmup, len(gaps))
