"""The CPU oracle against fixtures produced by the reference itself (tests/golden)."""
import numpy as np
import pytest

from oracle import ccsd as oc
from pycc_gb300.synth import SyntheticFactors


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_generator_matches_golden(golden_o5v19, ham_o5v19):
    fac = ham_o5v19[0]
    assert float(np.sum(fac.B * fac.B)) == pytest.approx(float(golden_o5v19["B_checksum"]), rel=1e-14)
    assert np.array_equal(fac.eps, golden_o5v19["eps"])


def test_intermediates_golden_o5v19(golden_o5v19, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    o, v = slice(0, 5), slice(5, 24)
    X = oc.intermediates(o, v, F, ERI, L, golden_o5v19["probe_t1"], golden_o5v19["probe_t2"])
    for k, val in X.items():
        assert rel(val, golden_o5v19[k]) < 1e-13, k
    assert rel(oc.build_tau(golden_o5v19["probe_t1"], golden_o5v19["probe_t2"]), golden_o5v19["tau"]) < 1e-14
    assert rel(oc.build_tau(golden_o5v19["probe_t1"], golden_o5v19["probe_t2"], 1.0, 0.5), golden_o5v19["taut"]) < 1e-14


def test_residuals_golden_o5v19(golden_o5v19, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    o, v = slice(0, 5), slice(5, 24)
    r1, r2 = oc.residuals(o, v, F, ERI, L, golden_o5v19["probe_t1"], golden_o5v19["probe_t2"])
    assert rel(r1, golden_o5v19["r1"]) < 1e-12
    assert rel(r2, golden_o5v19["r2"]) < 1e-12
    t1, t2 = oc.mp2_guess(F, ERI, 5)
    r1, r2 = oc.residuals(o, v, F, ERI, L, t1, t2)
    assert rel(r2, golden_o5v19["r2_mp2"]) < 1e-12
    assert np.abs(r1 - golden_o5v19["r1_mp2"]).max() < 1e-14
    assert oc.cc_energy(o, v, F, L, t1, t2) == pytest.approx(float(golden_o5v19["ecc_mp2"]), abs=1e-14)
    assert oc.cc_energy(o, v, F, L, golden_o5v19["probe_t1"], golden_o5v19["probe_t2"]) == pytest.approx(
        float(golden_o5v19["ecc_probe"]), abs=1e-13)


def test_solve_cc_golden_o5v19(golden_o5v19, ham_o5v19):
    _, F, ERI, L = ham_o5v19
    e, t1, t2, es = oc.solve_cc(F, ERI, L, 5, 1e-12, 1e-12)
    assert abs(e - float(golden_o5v19["ecc"])) < 1e-11
    assert len(es) == len(golden_o5v19["ecc_iters"])
    assert np.abs(np.array(es) - golden_o5v19["ecc_iters"]).max() < 1e-11
    assert rel(t2, golden_o5v19["t2"]) < 1e-9


def test_solve_cc_raises_on_maxiter(ham_o5v19):
    _, F, ERI, L = ham_o5v19
    with pytest.raises(RuntimeError):
        oc.solve_cc(F, ERI, L, 5, 1e-14, 1e-14, maxiter=3)


def probe_amplitudes(no, nv, t2_mp2, seed):
    """Same draw as tests/golden/make_golden.py:probe_amplitudes."""
    rng = np.random.default_rng(1000 + seed)
    t1 = 0.02 * rng.standard_normal((no, nv))
    noise = 0.01 * rng.standard_normal((no, no, nv, nv))
    return t1, t2_mp2 + noise + noise.transpose(1, 0, 3, 2)


def test_generator_o20v180_checksums():
    from conftest import golden
    for name, coupling in (("o20v180.npz", "matched"), ("o20v180_raw.npz", 1.0)):
        g = golden(name)
        fac = SyntheticFactors(20, 180, 1, coupling=coupling)
        assert float(np.sum(fac.B * fac.B)) == pytest.approx(float(g["B_checksum"]), rel=1e-13)


def test_residuals_o20v180_golden():
    """The oracle's residual at no=20, nv=180 against the reference's (about a minute)."""
    from conftest import golden
    g = golden("o20v180.npz")
    fac = SyntheticFactors(20, 180, 1, coupling="matched")
    F, ERI, L = fac.hamiltonian()
    o, v = slice(0, 20), slice(20, 200)
    t1, t2 = probe_amplitudes(20, 180, oc.mp2_guess(F, ERI, 20)[1], 1)
    r1, r2 = oc.residuals(o, v, F, ERI, L, t1, t2)
    assert rel(r1, g["r1"]) < 1e-12
    assert rel(r2[0, 1], g["r2_slice_ij01"]) < 1e-12
    assert rel(r2[:, :, 0, 0], g["r2_slice_ab00"]) < 1e-12
    assert np.linalg.norm(r2) == pytest.approx(float(g["r2_norm"]), rel=1e-12)


def test_triples_oracle_golden_o5v19(golden_o5v19, ham_o5v19):
    """The (T) oracle (Lee-Rendell over i >= j >= k, and the full-(i, j, k) X1/X2 form) on the
    reference's converged amplitudes against the reference's own t_tjl and t_vikings."""
    from oracle import triples as ot
    _, F, ERI, L = ham_o5v19
    t1, t2 = golden_o5v19["t1"], golden_o5v19["t2"]
    assert ot.t_tjl(5, 19, F, ERI, t1, t2) == pytest.approx(float(golden_o5v19["et_tjl"]), abs=1e-14)
    assert ot.t_vikings(5, 19, F, ERI, L, t1, t2) == pytest.approx(float(golden_o5v19["et_vikings"]),
                                                                    abs=1e-14)


def test_density_fixture_energy_identity(golden_o5v19, ham_o5v19):
    """The reference's gradient densities reproduce its correlation energy,
    E = <D, F> + <Gamma, ERI> (the identity of pycc/tests/test_076_ccsd_gradient.py:103-111):
    the D and Gamma fixtures the GPU adjoint is compared with are consistent."""
    _, F, ERI, _ = ham_o5v19
    E = float(np.sum(golden_o5v19["D"] * F) + np.sum(golden_o5v19["Gamma"] * ERI))
    assert E == pytest.approx(float(golden_o5v19["ecc"]), abs=1e-12)
    assert E == pytest.approx(float(golden_o5v19["E_from_densities"]), abs=1e-12)
