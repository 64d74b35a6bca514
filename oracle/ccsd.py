"""CPU oracle for the RHF-CCSD amplitude path -- TEST INFRASTRUCTURE ONLY.

A plain numpy restatement of the reference's spin-adapted closed-shell CCSD equations
(CrawfordGroup/pycc, ``pycc/ccwfn.py``) and its DIIS extrapolator (``pycc/utils.py``).
Each function cites the reference lines it follows.  Pairwise contractions go through
``numpy.einsum(..., optimize=True)``, which lowers them onto BLAS GEMMs as the reference's
``opt_einsum.contract`` does on the CPU (``pycc/device.py:64-70``).

This module is the checker of the CUDA engine in ``pycc_gb300``: only the test-suite,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it.  It is pinned
against fixtures produced by the reference itself (``tests/golden/make_golden.py``).

Index conventions follow the reference: ``t1[i,a]``, ``t2[i,j,a,b]``, ``ERI[p,q,r,s] =
<pq|rs>`` and ``L = 2 ERI - ERI.swapaxes(2,3)``; ``o``/``v`` are slices into the MO space.
"""
from __future__ import annotations

import numpy as np


def contract(subscripts, *ops):
    return np.einsum(subscripts, *ops, optimize=True)


class Blocks:
    """The o/v integral blocks the residual reads, as views of the full tensors."""

    def __init__(self, F, ERI, L, no):
        n = F.shape[0]
        o, v = slice(0, no), slice(no, n)
        self.no, self.nv = no, n - no
        self.F = F
        self.o, self.v = o, v
        self.ERI, self.L = ERI, L


# --- pycc/ccwfn.py:432-455 -------------------------------------------------------------
def build_tau(t1, t2, fact1=1.0, fact2=1.0):
    """tau_ijab = fact1 t2_ijab + fact2 t_ia t_jb  (ccwfn.py:454)."""
    return fact1 * t2 + fact2 * contract('ia,jb->ijab', t1, t1)


# --- pycc/ccwfn.py:458-498 -------------------------------------------------------------
def build_Fae(o, v, F, L, t1, t2):
    """F_ae (ccwfn.py:493-497)."""
    Fae = F[v, v].copy()
    Fae = Fae - 0.5 * contract('me,ma->ae', F[o, v], t1)
    Fae = Fae + contract('mf,mafe->ae', t1, L[o, v, v, v])
    Fae = Fae - contract('mnaf,mnef->ae', build_tau(t1, t2, 1.0, 0.5), L[o, o, v, v])
    return Fae


# --- pycc/ccwfn.py:501-534 -------------------------------------------------------------
def build_Fmi(o, v, F, L, t1, t2):
    """F_mi (ccwfn.py:529-533)."""
    Fmi = F[o, o].copy()
    Fmi = Fmi + 0.5 * contract('ie,me->mi', t1, F[o, v])
    Fmi = Fmi + contract('ne,mnie->mi', t1, L[o, o, o, v])
    Fmi = Fmi + contract('inef,mnef->mi', build_tau(t1, t2, 1.0, 0.5), L[o, o, v, v])
    return Fmi


# --- pycc/ccwfn.py:537-565 -------------------------------------------------------------
def build_Fme(o, v, F, L, t1):
    """F_me (ccwfn.py:562-564)."""
    return F[o, v] + contract('nf,mnef->me', t1, L[o, o, v, v])


# --- pycc/ccwfn.py:568-604 -------------------------------------------------------------
def build_Wmnij(o, v, ERI, t1, t2):
    """W_mnij (ccwfn.py:596-603)."""
    W = ERI[o, o, o, o].copy()
    W = W + contract('je,mnie->mnij', t1, ERI[o, o, o, v])
    W = W + contract('ie,mnej->mnij', t1, ERI[o, o, v, o])
    W = W + contract('ijef,mnef->mnij', build_tau(t1, t2), ERI[o, o, v, v])
    return W


# --- pycc/ccwfn.py:607-646 -------------------------------------------------------------
def build_Wmbej(o, v, ERI, L, t1, t2):
    """W_mbej (ccwfn.py:641-645)."""
    W = ERI[o, v, v, o].copy()
    W = W + contract('jf,mbef->mbej', t1, ERI[o, v, v, v])
    W = W - contract('nb,mnej->mbej', t1, ERI[o, o, v, o])
    W = W - contract('jnfb,mnef->mbej', build_tau(t1, t2, 0.5, 1.0), ERI[o, o, v, v])
    W = W + 0.5 * contract('njfb,mnef->mbej', t2, L[o, o, v, v])
    return W


# --- pycc/ccwfn.py:649-684 -------------------------------------------------------------
def build_Wmbje(o, v, ERI, t1, t2):
    """W_mbje (ccwfn.py:680-683)."""
    W = -1.0 * ERI[o, v, o, v]
    W = W - contract('jf,mbfe->mbje', t1, ERI[o, v, v, v])
    W = W + contract('nb,mnje->mbje', t1, ERI[o, o, o, v])
    W = W + contract('jnfb,mnfe->mbje', build_tau(t1, t2, 0.5, 1.0), ERI[o, o, v, v])
    return W


# --- pycc/ccwfn.py:687-715 -------------------------------------------------------------
def build_Zmbij(o, v, ERI, t1, t2):
    """Z_mbij (ccwfn.py:715)."""
    return contract('mbef,ijef->mbij', ERI[o, v, v, v], build_tau(t1, t2))


# --- pycc/ccwfn.py:718-761 -------------------------------------------------------------
def r_T1(o, v, F, ERI, L, t1, t2, Fae, Fme, Fmi):
    """Singles residual (ccwfn.py:753-760)."""
    r = F[v, o].swapaxes(0, 1).copy()
    r = r + contract('ie,ae->ia', t1, Fae)
    r = r - contract('mi,ma->ia', Fmi, t1)
    t2s = 2.0 * t2 - t2.swapaxes(2, 3)
    r = r + contract('imae,me->ia', t2s, Fme)
    r = r + contract('nf,nafi->ia', t1, L[o, v, v, o])
    r = r + contract('mief,maef->ia', t2s, ERI[o, v, v, v])
    r = r - contract('mnae,nmei->ia', t2, L[o, o, v, o])
    return r


# --- pycc/ccwfn.py:764-791 and :886-945 ----------------------------------------------
def r_T2_half(o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
    """Doubles residual before the i<->j / a<->b symmetrisation (ccwfn.py:922-940)."""
    r = 0.5 * ERI[v, v, o, o].transpose(2, 3, 0, 1).copy()
    r = r + contract('ijae,eb->ijab', t2, Fae.T)
    tmp = contract('bm,me->be', t1.T, Fme)
    r = r - 0.5 * contract('ijae,eb->ijab', t2, tmp.T)
    r = r - contract('imab,mj->ijab', t2, Fmi)
    tmp = contract('je,em->jm', t1, Fme.T)
    r = r - 0.5 * contract('imab,mj->ijab', t2, tmp.T)
    tau = build_tau(t1, t2)
    r = r + 0.5 * contract('mnab,mnij->ijab', tau, Wmnij)
    r = r + 0.5 * contract('ijef,abef->ijab', tau, ERI[v, v, v, v])
    r = r - contract('ma,mbij->ijab', t1, Zmbij)
    r = r + contract('imae,mbej->ijab', t2 - t2.swapaxes(2, 3), Wmbej)
    r = r + contract('imae,mbej->ijab', t2, Wmbej + Wmbje.swapaxes(2, 3))
    r = r + contract('mjae,mbie->ijab', t2, Wmbje)
    tmp = contract('ei,am->aemi', t1.T, t1.T).transpose(3, 2, 1, 0)   # [i,m,e,a] = t_ie t_ma
    r = r - contract('imea,mbej->ijab', tmp, ERI[o, v, v, o])
    r = r - contract('imeb,maje->ijab', tmp, ERI[o, v, o, v])
    r = r + contract('ie,abej->ijab', t1, ERI[v, v, v, o])
    r = r - contract('ma,mbij->ijab', t1, ERI[o, v, o, o])
    return r


def r_T2(o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
    """Symmetrised doubles residual (ccwfn.py:789-790)."""
    r = r_T2_half(o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij)
    return r + r.swapaxes(0, 1).swapaxes(2, 3)


# --- pycc/ccwfn.py:321-372 -------------------------------------------------------------
def intermediates(o, v, F, ERI, L, t1, t2):
    """All one- and two-body intermediates in the order residuals() builds them (:350-356)."""
    return dict(
        Fae=build_Fae(o, v, F, L, t1, t2),
        Fmi=build_Fmi(o, v, F, L, t1, t2),
        Fme=build_Fme(o, v, F, L, t1),
        Wmnij=build_Wmnij(o, v, ERI, t1, t2),
        Wmbej=build_Wmbej(o, v, ERI, L, t1, t2),
        Wmbje=build_Wmbje(o, v, ERI, t1, t2),
        Zmbij=build_Zmbij(o, v, ERI, t1, t2),
    )


def residuals(o, v, F, ERI, L, t1, t2):
    """(r1, r2) = residuals(F, t1, t2)  (ccwfn.py:350-359)."""
    X = intermediates(o, v, F, ERI, L, t1, t2)
    r1 = r_T1(o, v, F, ERI, L, t1, t2, X["Fae"], X["Fme"], X["Fmi"])
    r2 = r_T2(o, v, F, ERI, t1, t2, X["Fae"], X["Fme"], X["Fmi"], X["Wmnij"],
              X["Wmbej"], X["Wmbje"], X["Zmbij"])
    return r1, r2


# --- pycc/ccwfn.py:1122-1162 -----------------------------------------------------------
def cc_energy(o, v, F, L, t1, t2):
    """E = 2 f_ia t_ia + tau_ijab L_ijab  (ccwfn.py:1159-1161)."""
    e = 2.0 * contract('ia,ia->', F[o, v], t1)
    return float(e + contract('ijab,ijab->', build_tau(t1, t2), L[o, o, v, v]))


# --- pycc/utils.py:257-361 -------------------------------------------------------------
class DIIS:
    """Pulay DIIS on the amplitude differences e_n = t_n - t_{n-1} (utils.py:272-361)."""

    def __init__(self, t1, t2, max_diis):
        self.old1, self.old2 = t1.copy(), t2.copy()
        self.vals1, self.vals2 = [t1.copy()], [t2.copy()]
        self.errors = []
        self.max_diis = max_diis

    def add_error_vector(self, t1, t2):
        """utils.py:284-295."""
        self.vals1.append(t1.copy())
        self.vals2.append(t2.copy())
        self.errors.append(np.concatenate(((t1 - self.old1).ravel(), (t2 - self.old2).ravel())))
        self.old1, self.old2 = t1.copy(), t2.copy()

    def extrapolate(self, t1, t2):
        """utils.py:297-361: bordered B, max-abs scaling, Pulay solve, combination."""
        if self.max_diis == 0:
            return t1, t2
        if len(self.errors) > self.max_diis:
            del self.vals1[0]
            del self.vals2[0]
            del self.errors[0]
        k = len(self.errors)
        B = -np.ones((k + 1, k + 1))
        B[-1, -1] = 0.0
        for a in range(k):
            for b in range(a, k):
                B[a, b] = B[b, a] = np.dot(self.errors[a], self.errors[b])
        B[:-1, :-1] /= np.abs(B[:-1, :-1]).max()
        rhs = np.zeros(k + 1)
        rhs[-1] = -1.0
        c = np.linalg.solve(B, rhs)
        t1 = np.zeros_like(self.old1)
        t2 = np.zeros_like(self.old2)
        for n in range(k):
            t1 += c[n] * self.vals1[n + 1]
            t2 += c[n] * self.vals2[n + 1]
        self.old1, self.old2 = t1.copy(), t2.copy()
        return t1, t2


# --- pycc/ccwfn.py:195-211, :216-319 ---------------------------------------------------
def denominators(F, no):
    eps = np.diag(F)
    eo, ev = eps[:no], eps[no:]
    Dia = eo.reshape(-1, 1) - ev
    Dijab = eo.reshape(-1, 1, 1, 1) + eo.reshape(-1, 1, 1) - ev.reshape(-1, 1) - ev
    return Dia, Dijab


def mp2_guess(F, ERI, no):
    """t1 = 0, t2 = <ij|ab>/D_ijab (ccwfn.py:209-211)."""
    n = F.shape[0]
    o, v = slice(0, no), slice(no, n)
    Dia, Dijab = denominators(F, no)
    return np.zeros((no, n - no)), ERI[o, o, v, v] / Dijab


def solve_cc(F, ERI, L, no, e_conv=1e-7, r_conv=1e-7, maxiter=100, max_diis=8, start_diis=1,
             t1=None, t2=None, callback=None):
    """Jacobi + DIIS iteration of solve_cc (ccwfn.py:260-319).

    Returns ``(ecc, t1, t2, energies)``; ``energies[0]`` is the guess energy.  Raises
    ``RuntimeError`` when ``maxiter`` is exhausted (the reference falls through and
    returns ``None`` there).
    """
    n = F.shape[0]
    o, v = slice(0, no), slice(no, n)
    Dia, Dijab = denominators(F, no)
    if t1 is None:
        t1, t2 = mp2_guess(F, ERI, no)
    t1, t2 = t1.copy(), t2.copy()
    ecc = cc_energy(o, v, F, L, t1, t2)
    energies = [ecc]
    diis = DIIS(t1, t2, max_diis)
    for niter in range(1, maxiter + 1):
        ecc_last = ecc
        r1, r2 = residuals(o, v, F, ERI, L, t1, t2)
        t1 = t1 + r1 / Dia
        t2 = t2 + r2 / Dijab
        rms = np.sqrt(np.sum((r1 / Dia) ** 2) + np.sum((r2 / Dijab) ** 2))
        ecc = cc_energy(o, v, F, L, t1, t2)
        energies.append(ecc)
        if callback is not None:
            callback(niter, ecc, rms)
        if abs(ecc - ecc_last) < e_conv and rms < r_conv:
            return ecc, t1, t2, energies
        diis.add_error_vector(t1, t2)
        if niter >= start_diis:
            t1, t2 = diis.extrapolate(t1, t2)
    raise RuntimeError("CCSD did not converge in %d iterations" % maxiter)
