"""Generate the golden fixtures of the RHF-CCSD path by running the reference itself.

The reference (CrawfordGroup/pycc) is pure Python.  Its integral source needs psi4 and
qcelemental, which are not installed, but the CCSD arithmetic never touches them: this
script puts inert stand-ins for both modules into ``sys.modules``, imports ``pycc`` from
the reference tree named by ``$PYCC_REF`` (required), and assembles a ``CCwfn``
with ``CCwfn.__new__`` plus the attributes that ``CCwfn.__init__`` would have set
(``pycc/ccwfn.py:76-213``, ``pycc/wavefunction.py:293-332``), on the synthetic
Hamiltonian of ``pycc_gb300.synth``.  It then runs the reference's own
``residuals`` / ``solve_cc`` / ``t_vikings`` / ``t_tjl`` / ``cchbar`` -> ``cclambda``
-> ``ccdensity`` / ``CCderiv._ccsd_jacobian`` and the complex residual, and stores their outputs as ``.npz`` fixtures next to this file.

Usage::

    PYCC_REF=<reference tree> PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [--o20v180] [--no-o5v19] [--no-jacobian] [--no-complex] [--no-hbar] [--no-t3density]

The no=20, nv=180 fixtures need ~30 GB of host RAM and several minutes.
"""
from __future__ import annotations

import argparse
import io
import contextlib
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pycc_gb300.synth import SyntheticFactors, WORKLOADS  # noqa: E402
from oracle import reference as _ref  # noqa: E402


def import_reference():
    """The reference package from ``$PYCC_REF`` (its source tree), with psi4 / qcelemental
    stand-ins (``oracle.reference.import_reference``)."""
    ref = os.environ.get("PYCC_REF")
    if not ref:
        raise SystemExit("make_golden.py: set PYCC_REF to the reference's source tree")
    return _ref.import_reference(ref)


make_ref_ccwfn = _ref.make_ref_ccwfn


def probe_amplitudes(no, nv, t2_mp2, seed):
    """A non-trivial (t1, t2) pair: every singles term of the residual is exercised."""
    rng = np.random.default_rng(1000 + seed)
    t1 = 0.02 * rng.standard_normal((no, nv))
    noise = 0.01 * rng.standard_normal((no, no, nv, nv))
    noise = noise + noise.transpose(1, 0, 3, 2)       # keep t2_ijab = t2_jiba
    t2 = t2_mp2 + noise
    return t1, t2


def quiet(fn, *args, **kwargs):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*args, **kwargs)


def gen_o5v19(pycc):
    no, nv, seed = WORKLOADS["o5v19"]
    fac = SyntheticFactors(no, nv, seed)
    F, ERI, L = fac.hamiltonian()
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    o, v = w.o, w.v
    out = {"no": no, "nv": nv, "seed": seed, "B_checksum": float(np.sum(fac.B * fac.B)),
           "eps": fac.eps}
    # residual + intermediates at a probe point with non-zero singles
    t1, t2 = probe_amplitudes(no, nv, w.t2, seed)
    out["probe_t1"], out["probe_t2"] = t1, t2
    out["tau"] = w.build_tau(t1, t2)
    out["taut"] = w.build_tau(t1, t2, 1.0, 0.5)
    out["Fae"] = w.build_Fae(o, v, F, L, t1, t2)
    out["Fmi"] = w.build_Fmi(o, v, F, L, t1, t2)
    out["Fme"] = w.build_Fme(o, v, F, L, t1)
    out["Wmnij"] = w.build_Wmnij(o, v, ERI, t1, t2)
    out["Wmbej"] = w.build_Wmbej(o, v, ERI, L, t1, t2)
    out["Wmbje"] = w.build_Wmbje(o, v, ERI, t1, t2)
    out["Zmbij"] = w.build_Zmbij(o, v, ERI, t1, t2)
    r1, r2 = w.residuals(F, t1, t2)
    out["r1"], out["r2"] = r1, r2
    out["ecc_probe"] = float(w.cc_energy(o, v, F, L, t1, t2))
    # residual at the MP2 guess
    r1m, r2m = w.residuals(F, w.t1, w.t2)
    out["r1_mp2"], out["r2_mp2"] = r1m, r2m
    out["ecc_mp2"] = float(w.cc_energy(o, v, F, L, w.t1, w.t2))
    # converged CCSD, recording every iteration's energy
    energies = []
    orig = w.cc_energy

    def rec(*a):
        e = orig(*a)
        energies.append(float(e))
        return e
    w.cc_energy = rec
    ecc = quiet(w.solve_cc, 1e-12, 1e-12, 100, 8, 1)
    del w.cc_energy
    out["ecc"] = float(ecc)
    out["ecc_iters"] = np.array(energies)
    out["t1"], out["t2"] = w.t1, w.t2
    # (T): the vectorised and the Lee-Rendell drivers
    from pycc.cctriples import t_vikings, t_tjl
    out["et_vikings"] = float(t_vikings(w))
    out["et_tjl"] = float(t_tjl(w))
    # Lambda and the gradient densities
    from pycc.cchbar import cchbar
    from pycc.cclambda import cclambda
    from pycc.ccdensity import ccdensity
    hbar = quiet(cchbar, w)
    lam = quiet(cclambda, w, hbar)
    pseudo = quiet(lam.solve_lambda, 1e-12, 1e-12, 100, 8, 1)
    out["lambda_pseudo"] = float(pseudo)
    out["l1"], out["l2"] = lam.l1, lam.l2
    dens = quiet(ccdensity, w, lam)
    D, G = quiet(dens.gradient_densities)
    out["D"] = np.asarray(D)
    out["Gamma"] = np.asarray(G)
    out["E_from_densities"] = float(np.sum(D * F) + np.sum(G * ERI))
    np.savez_compressed(os.path.join(HERE, "o5v19.npz"), **out)
    print("golden_o5v19: ecc = %.15f  (T) = %.15f / %.15f  pseudo = %.15f  E(D,G) = %.15f  niter = %d"
          % (ecc, out["et_vikings"], out["et_tjl"], pseudo, out["E_from_densities"],
             len(energies) - 1))


def gen_o5v19_jacobian(pycc):
    """The reference's CCSD Jacobian action at the converged no=5, nv=19 amplitudes:
    ``CCderiv._ccsd_jacobian(X1, X2, hbar)`` (pycc/ccderiv.py:149-180) on a seeded amplitude
    pair X (X2_ijab = X2_jiba), called with the two attributes it reads (``contract`` and
    ``ccwfn``) instead of a full CCderiv, whose set-up needs psi4."""
    no, nv, seed = WORKLOADS["o5v19"]
    fac = SyntheticFactors(no, nv, seed)
    F, ERI, L = fac.hamiltonian()
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    ecc = quiet(w.solve_cc, 1e-12, 1e-12, 100, 8, 1)
    from pycc.cchbar import cchbar
    from pycc.ccderiv import CCderiv
    hbar = quiet(cchbar, w)
    rng = np.random.default_rng(2000 + seed)
    X1 = 0.1 * rng.standard_normal((no, nv))
    X2 = 0.1 * rng.standard_normal((no, no, nv, nv))
    X2 = X2 + X2.transpose(1, 0, 3, 2)
    host = types.SimpleNamespace(contract=w.contract, ccwfn=w)
    s1, s2 = CCderiv._ccsd_jacobian(host, X1, X2, hbar)
    out = {"ecc": float(ecc), "t1": w.t1, "t2": w.t2, "X1": X1, "X2": X2,
           "sigma1": np.asarray(s1), "sigma2": np.asarray(s2),
           "sigma2_sym": np.asarray(s2) + np.asarray(s2).transpose(1, 0, 3, 2)}
    np.savez_compressed(os.path.join(HERE, "o5v19_jacobian.npz"), **out)
    print("o5v19_jacobian: |sigma1| = %.6e  |sigma2_sym| = %.6e"
          % (np.linalg.norm(out["sigma1"]), np.linalg.norm(out["sigma2_sym"])))


def gen_o5v19_hbar(pycc):
    """The reference's eleven HBAR blocks (``cchbar.__init__``, pycc/cchbar.py:54-110) at its
    converged no=5, nv=19 amplitudes, and those amplitudes."""
    no, nv, seed = WORKLOADS["o5v19"]
    fac = SyntheticFactors(no, nv, seed)
    F, ERI, L = fac.hamiltonian()
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    ecc = quiet(w.solve_cc, 1e-12, 1e-12, 100, 8, 1)
    from pycc.cchbar import cchbar
    hbar = quiet(cchbar, w)
    names = ("Hov", "Hvv", "Hoo", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov", "Hvvvo",
             "Hovoo")
    out = {"ecc": float(ecc), "t1": w.t1, "t2": w.t2}
    for n in names:
        out[n] = np.asarray(getattr(hbar, n))
    np.savez_compressed(os.path.join(HERE, "o5v19_hbar.npz"), **out)
    print("o5v19_hbar: " + "  ".join("|%s| = %.6e" % (n, np.linalg.norm(out[n])) for n in names))


def gen_o5v19_t3density(pycc):
    """The reference's (T) densities and Lambda sources (``t3_density``,
    pycc/cctriples.py:1063-1157) at its converged no=5, nv=19 amplitudes."""
    no, nv, seed = WORKLOADS["o5v19"]
    fac = SyntheticFactors(no, nv, seed)
    F, ERI, L = fac.hamiltonian()
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    quiet(w.solve_cc, 1e-12, 1e-12, 100, 8, 1)
    from pycc.cctriples import t3_density
    et, dens = t3_density(w.o, w.v, no, nv, w.t1, w.t2, F, ERI, L, w.contract)
    out = {"et": float(et), "t1": w.t1, "t2": w.t2}
    out.update({k: np.asarray(x) for k, x in dens.items()})
    np.savez_compressed(os.path.join(HERE, "o5v19_t3density.npz"), **out)
    print("o5v19_t3density: E(T) = %.15f  " % et
          + "  ".join("|%s| = %.6e" % (k, np.linalg.norm(x)) for k, x in dens.items()))


def gen_o5v19_complex(pycc):
    """The reference's residual at complex amplitudes and a complex Fock matrix, as its
    real-time propagation calls it (``residuals(F, t1, t2, real_time=True)``): no=5, nv=19,
    seeded complex t1 / t2 (t2_ijab = t2_jiba) and F + i dF with a real symmetric dF."""
    no, nv, seed = WORKLOADS["o5v19"]
    fac = SyntheticFactors(no, nv, seed)
    F, ERI, L = fac.hamiltonian()
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    rng = np.random.default_rng(3000 + seed)
    t1 = 0.05 * (rng.standard_normal((no, nv)) + 1j * rng.standard_normal((no, nv)))
    t2 = 0.05 * (rng.standard_normal((no, no, nv, nv)) + 1j * rng.standard_normal((no, no, nv, nv)))
    t2 = t2 + t2.transpose(1, 0, 3, 2)
    dF = rng.standard_normal(F.shape)
    Fc = F + 0.01j * (dF + dF.T)
    r1, r2 = w.residuals(Fc, t1, t2, real_time=True)
    np.savez_compressed(os.path.join(HERE, "o5v19_complex.npz"), F=Fc, t1=t1, t2=t2,
                        r1=np.asarray(r1), r2=np.asarray(r2))
    print("o5v19_complex: |r1| = %.6e  |r2| = %.6e" % (np.linalg.norm(r1), np.linalg.norm(r2)))


def gen_o20v180(pycc, solve=True, coupling="matched", name="o20v180.npz"):
    """no=20, nv=180, seed 1.  With the spec's plain sigma (coupling 1) CCSD diverges at this
    size, so the converged fixture uses the matched coupling; the raw-sigma fixture keeps the
    residual at the probe point only."""
    no, nv, seed = WORKLOADS["o20v180"]
    fac = SyntheticFactors(no, nv, seed, coupling=coupling)
    t0 = time.time()
    F, ERI, L = fac.hamiltonian()
    print("o20v180: integrals %.1f s" % (time.time() - t0), flush=True)
    w = make_ref_ccwfn(pycc, F, ERI, L, no, nv)
    o, v = w.o, w.v
    out = {"no": no, "nv": nv, "seed": seed, "B_checksum": float(np.sum(fac.B * fac.B)),
           "coupling": fac.coupling}
    t1, t2 = probe_amplitudes(no, nv, w.t2, seed)
    t0 = time.time()
    r1, r2 = w.residuals(F, t1, t2)
    print("o20v180: residual %.1f s" % (time.time() - t0), flush=True)
    out["r1"] = r1
    out["r2_norm"] = float(np.linalg.norm(r2))
    out["r2_slice_ij01"] = r2[0, 1].copy()
    out["r2_slice_ab00"] = r2[:, :, 0, 0].copy()
    out["r2_slice_diag"] = r2[3, 3, 10:20, 100:110].copy()
    out["r2_rowsum"] = r2.sum(axis=(2, 3))
    out["ecc_probe"] = float(w.cc_energy(o, v, F, L, t1, t2))
    if solve:
        energies = []
        orig = w.cc_energy

        def rec(*a):
            e = orig(*a)
            energies.append(float(e))
            return e
        w.cc_energy = rec
        t0 = time.time()
        ecc = quiet(w.solve_cc, 1e-10, 1e-10, 100, 8, 1)
        print("o20v180: solve %.1f s, %d iterations" % (time.time() - t0, len(energies) - 1))
        out["ecc"] = float(ecc)
        out["ecc_iters"] = np.array(energies)
        out["t1"] = w.t1
        out["t2_norm"] = float(np.linalg.norm(w.t2))
        out["t2_slice_ij01"] = w.t2[0, 1].copy()
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("o20v180: done", name, out.get("ecc"), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--o20v180", action="store_true")
    ap.add_argument("--no-o5v19", action="store_true")
    ap.add_argument("--no-jacobian", action="store_true")
    ap.add_argument("--no-complex", action="store_true")
    ap.add_argument("--no-hbar", action="store_true")
    ap.add_argument("--no-t3density", action="store_true")
    args = ap.parse_args()
    pycc = import_reference()
    if not args.no_o5v19:
        gen_o5v19(pycc)
    if not args.no_jacobian:
        gen_o5v19_jacobian(pycc)
    if not args.no_complex:
        gen_o5v19_complex(pycc)
    if not args.no_hbar:
        gen_o5v19_hbar(pycc)
    if not args.no_t3density:
        gen_o5v19_t3density(pycc)
    if args.o20v180:
        gen_o20v180(pycc, solve=False, coupling=1.0, name="o20v180_raw.npz")
        gen_o20v180(pycc, solve=True, coupling="matched", name="o20v180.npz")


if __name__ == "__main__":
    main()
