"""Seeded synthetic canonical-MO Hamiltonians for the RHF-CCSD engine.

The generator stands in for a psi4 SCF + MO integral transform (the reference builds
``H.F``, ``H.ERI`` and ``H.L`` in ``pycc/hamiltonian.py:36-70``).  It keeps the reference's
data layout exactly:

* ``F``   : (nmo, nmo) diagonal Fock matrix, occupied block first;
* ``ERI`` : physicist ``<pq|rs> = (pr|qs)`` (``pycc/hamiltonian.py:67-69``);
* ``L``   : ``2 <pq|rs> - <pq|sr>`` (``pycc/hamiltonian.py:70``).

Draw order (fixed so that every consumer sees the same arrays)::

    rng   = numpy.random.default_rng(seed)
    eps_o = sort(rng.uniform(-1.2, -0.4, no))
    eps_v = sort(rng.uniform( 0.3,  2.5, nv))
    B[Q, p, q>=p] = rng.normal(0, 0.35/sqrt(naux)), row-major over (Q, p, q>=p),
                    mirrored so that B[Q, q, p] = B[Q, p, q];  naux = 3 * nmo
    (pq|rs) = sum_Q B[Q,p,q] B[Q,r,s]

The chemist tensor is positive semi-definite with full 8-fold permutational symmetry.

Coupling scale.  With the plain sigma above, the pair-coupling strength
``o^2 v^2 var(<ij|ab>) ~ o^2 v^2 (0.35^2)^2 / naux`` grows with the size: at no=5, nv=19 the
CCSD energy is -0.73 Eh and the iteration converges, but at no=20, nv=180 the MP2 energy
is already about -160 Eh and the CCSD iteration diverges (for the reference and for this
engine alike).  ``coupling`` multiplies sigma by lambda; ``coupling='matched'`` picks
lambda = (125.35 naux / (o^2 v^2))^(1/4), which keeps o^2 v^2 var(<ij|ab>) at its
no=5, nv=19 value (lambda = 1 there exactly) so every size is a convergent, moderately
correlated problem.  The draw order and every other distribution are unchanged.
The full ``nmo^4`` tensors are only built on the host for small sizes; large problems
build the needed ``o/v`` blocks on the GPU from ``B`` (see ``pycc_gb300.hamiltonian``).
"""
from __future__ import annotations

import numpy as np

#: The synthetic workloads of the RHF-CCSD engine, named by size: (no, nv, seed).
#: o5v19 is small enough for the reference itself (the golden vectors); o20v180 is the
#: largest the reference's host arrays hold; o40v300 is the CCSD benchmark; o20v180s3 the
#: adjoint measurement; o30v240 the (T) measurement.
WORKLOADS = {
    "o5v19": (5, 19, 0),
    "o20v180": (20, 180, 1),
    "o40v300": (40, 300, 2),
    "o20v180s3": (20, 180, 3),
    "o30v240": (30, 240, 4),
}


class SyntheticFactors:
    """Orbital energies and the symmetric 3-index factor ``B[Q,p,q]`` of one Hamiltonian."""

    def __init__(self, no: int, nv: int, seed: int, naux: int | None = None, coupling=1.0):
        self.no = int(no)
        self.nv = int(nv)
        self.nmo = self.no + self.nv
        self.naux = int(naux) if naux is not None else 3 * self.nmo
        self.seed = int(seed)
        if coupling == "matched":
            coupling = matched_coupling(self.no, self.nv, self.naux)
        self.coupling = float(coupling)
        n = self.nmo
        rng = np.random.default_rng(self.seed)
        eps_o = np.sort(rng.uniform(-1.2, -0.4, self.no))
        eps_v = np.sort(rng.uniform(0.3, 2.5, self.nv))
        self.eps = np.concatenate((eps_o, eps_v))
        sigma = self.coupling * 0.35 / np.sqrt(self.naux)
        iu = np.triu_indices(n)
        draws = rng.normal(0.0, sigma, size=(self.naux, iu[0].size))
        B = np.empty((self.naux, n, n))
        B[:, iu[0], iu[1]] = draws
        B[:, iu[1], iu[0]] = draws
        self.B = B

    @property
    def F(self) -> np.ndarray:
        return np.diag(self.eps)

    def chemist(self) -> np.ndarray:
        """Full ``(pq|rs)`` (nmo^4, float64).  Host memory: 8 nmo^4 bytes."""
        n, naux = self.nmo, self.naux
        Bm = self.B.reshape(naux, n * n)
        out = np.empty((n * n, n * n))
        step = 2048                       # row blocks keep each GEMM call moderate
        for r0 in range(0, n * n, step):
            r1 = min(n * n, r0 + step)
            out[r0:r1] = Bm[:, r0:r1].T @ Bm
        return out.reshape(n, n, n, n)

    def eri(self) -> np.ndarray:
        """Full physicist ``<pq|rs> = (pr|qs)`` as a C-contiguous array."""
        return np.ascontiguousarray(self.chemist().transpose(0, 2, 1, 3))

    def hamiltonian(self):
        """Return ``(F, ERI, L)`` on the host, in the reference's layout."""
        ERI = self.eri()
        L = 2.0 * ERI
        L -= ERI.swapaxes(2, 3)
        return self.F, ERI, L


#: o^2 v^2 / naux at no=5, nv=19 (naux=72): the coupling strength 'matched' keeps.
_REF_STRENGTH = (5 * 5 * 19 * 19) / 72.0


def matched_coupling(no: int, nv: int, naux: int) -> float:
    """lambda with lambda^4 o^2 v^2 / naux equal to its no=5, nv=19 value."""
    if (no, nv, naux) == (5, 19, 72):
        return 1.0
    return float((_REF_STRENGTH * naux / float(no * no * nv * nv)) ** 0.25)


def synthetic_factors(name: str, coupling=1.0) -> SyntheticFactors:
    no, nv, seed = WORKLOADS[name]
    return SyntheticFactors(no, nv, seed, coupling=coupling)
