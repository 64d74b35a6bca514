"""Host logic of the GPU DIIS (``pycc_gb300.diis``), on CPU.

The library's vector entry points are replaced by a numpy model of their documented
semantics (``pcg_diis_error_f64/f32``: e = x - old, out[j] = <e, ys[j]>, out[k-1] = <e, e>;
``pcg_lincomb_f64/_df``: out = sum_j c_j xs[j]) that also enforces their limit of 16 vectors
per call and the no-alias rule.  Tensors live in host memory, so ``data_ptr()`` addresses
are readable here.  The DIIS history is checked against the oracle's restatement of
helper_diis (pycc/utils.py:257-361) where it outgrows one call:

* ``start_diis`` past the window: the reference trims one vector per extrapolation
  (utils.py:322-326), so its history stays longer than ``max_diis``;
* ``max_diis`` above 15;
* ``max_diis == 0`` (extrapolation off, utils.py:318-319): no history and no library calls.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pycc_gb300 import _lib, diis as diis_mod
from pycc_gb300.diis import DIIS
from oracle import ccsd as oc


def _view(ptr, n, dtype):
    dt = np.dtype(dtype)
    return np.frombuffer((C.c_char * (n * dt.itemsize)).from_address(ptr), dtype=dt)


class FakeLib:
    """numpy model of the DIIS entry points on host memory."""

    def __init__(self, limit=16):
        self.limit = limit
        self.calls = []

    def __call__(self, name, *a):
        if name.startswith("pcg_diis_error_"):
            x, old, e, ys, k, n, _work, _wl, out, _st = a
            self._check(name, k)
            dt = np.float32 if name.endswith("f32") else np.float64
            E = _view(e, n, dt)
            E[:] = (_view(x, n, np.float64) - _view(old, n, np.float64)).astype(dt)
            e64 = E.astype(np.float64)
            o = _view(out, k, np.float64)
            for j in range(k - 1):
                o[j] = np.dot(e64, _view(ys[j], n, dt).astype(np.float64))
            o[k - 1] = np.dot(e64, e64)
        elif name.startswith("pcg_lincomb_"):
            xs, c, k, n, out, _st = a
            self._check(name, k)
            assert all(xs[j] != out for j in range(k)), "output aliases an input"
            acc = np.zeros(n)
            for j in range(k):
                acc = acc + c[j] * _view(xs[j], n, np.float64)
            _view(out, n, np.float64)[:] = acc
        else:
            raise AssertionError("unexpected entry point %s" % name)
        self.calls.append((name, k))
        return 0

    def _check(self, name, k):
        if not 1 <= k <= self.limit:
            raise _lib.EngineError("%s: k=%d outside [1, %d]" % (name, k, self.limit))


@pytest.fixture
def fake(monkeypatch):
    f = FakeLib()
    monkeypatch.setattr(_lib, "call", f)
    monkeypatch.setattr(_lib, "stream_handle", lambda stream=None: None)
    return f


def _sequence(n1, n2, steps, seed):
    rng = np.random.default_rng(seed)
    t1s, t2s = [rng.standard_normal(n1) * 0.05], [rng.standard_normal(n2) * 0.01]
    lim1, lim2 = rng.standard_normal(n1) * 0.05, rng.standard_normal(n2) * 0.01
    for s in range(steps):
        f = 0.7 ** (s + 1)
        t1s.append(lim1 + f * (t1s[0] - lim1) + 1e-3 * f * rng.standard_normal(n1))
        t2s.append(lim2 + f * (t2s[0] - lim2) + 1e-3 * f * rng.standard_normal(n2))
    return t1s, t2s


def _run(t1s, t2s, max_diis, start_diis, error_dtype=torch.float64):
    """Feed the iterates as the solver does (add, then extrapolate from start_diis)."""
    amps = torch.from_numpy(np.concatenate([t1s[0], t2s[0]]))
    d = DIIS(amps, max_diis, error_dtype=error_dtype)
    out = []
    for n, (a, b) in enumerate(zip(t1s[1:], t2s[1:]), start=1):
        amps = torch.from_numpy(np.concatenate([a, b]))
        d.add_error_vector(amps)
        if n >= start_diis:
            amps = d.extrapolate(amps)
        out.append(amps.numpy().copy())
    return d, out


def _oracle(t1s, t2s, max_diis, start_diis):
    ref = oc.DIIS(t1s[0], t2s[0], max_diis)
    out = []
    for n, (a, b) in enumerate(zip(t1s[1:], t2s[1:]), start=1):
        ref.add_error_vector(a, b)
        if n >= start_diis:
            a, b = ref.extrapolate(a, b)
        out.append(np.concatenate([a, b]))
    return out


@pytest.mark.parametrize("max_diis,start_diis,steps", [(8, 20, 26), (20, 1, 24), (8, 1, 12)])
def test_long_histories_match_oracle(fake, max_diis, start_diis, steps):
    t1s, t2s = _sequence(7, 61, steps, max_diis * 100 + start_diis)
    d, got = _run(t1s, t2s, max_diis, start_diis)
    want = _oracle(t1s, t2s, max_diis, start_diis)
    for g, w in zip(got, want):
        assert np.abs(g - w).max() <= 1e-12 * np.abs(w).max()
    assert max(k for _, k in fake.calls) <= 16
    longest = max(max_diis, start_diis - 1)
    assert len(d.errors) == min(longest, steps)
    if longest >= 16:                                  # chunked passes did happen
        assert sum(1 for name, _ in fake.calls if name.startswith("pcg_diis_error")) > steps


@pytest.mark.parametrize("error_dtype", [torch.float64, torch.float32])
def test_chunking_does_not_change_results(monkeypatch, error_dtype):
    """The same history run with one call per step (a limit of 64 vectors) and in chunks of
    16 gives the same overlaps and amplitudes up to the rounding of the partial sums."""
    monkeypatch.setattr(_lib, "stream_handle", lambda stream=None: None)
    t1s, t2s = _sequence(5, 40, 22, 11)
    results = []
    for limit in (64, 16):
        monkeypatch.setattr(_lib, "call", FakeLib(limit))
        monkeypatch.setattr(diis_mod, "MAX_VEC", limit)
        results.append(_run(t1s, t2s, 30, 1, error_dtype))
    (d0, a0), (d1, a1) = results
    assert np.array_equal(d0.B, d1.B)
    for u, v in zip(a0, a1):
        assert np.abs(u - v).max() <= 1e-14 * np.abs(u).max()


def test_max_diis_zero_keeps_no_history(fake):
    t1s, t2s = _sequence(4, 30, 40, 5)
    d, got = _run(t1s, t2s, 0, 1)
    for g, a, b in zip(got, t1s[1:], t2s[1:]):
        assert np.array_equal(g, np.concatenate([a, b]))
    assert fake.calls == [] and d.errors == [] and d.vals == []


def test_negative_max_diis_rejected():
    with pytest.raises(ValueError):
        DIIS(torch.zeros(4, dtype=torch.float64), -1)


@pytest.mark.parametrize("max_diis,start", [(8, 1), (3, 2), (0, 1)])
def test_helper_diis_interface(fake, max_diis, start):
    """pycc_gb300.utils.helper_diis keeps the reference's interface -- separate t1 / t2,
    add_error_vector(t1, t2), extrapolate(t1, t2) -> (t1, t2) -- and its results."""
    from pycc_gb300.utils import helper_diis
    t1s, t2s = _sequence(6, 50, 12, max_diis + 10 * start)
    sh1, sh2 = (3, 2), (5, 10)
    d = helper_diis(torch.from_numpy(t1s[0].reshape(sh1)), torch.from_numpy(t2s[0].reshape(sh2)),
                    max_diis)
    ref = oc.DIIS(t1s[0], t2s[0], max_diis)
    for n, (a, b) in enumerate(zip(t1s[1:], t2s[1:]), start=1):
        ta, tb = torch.from_numpy(a.reshape(sh1)), torch.from_numpy(b.reshape(sh2))
        d.add_error_vector(ta, tb)
        ref.add_error_vector(a, b)
        if n >= start:
            ga, gb = d.extrapolate(ta, tb)
            wa, wb = ref.extrapolate(a, b)
            assert tuple(ga.shape) == sh1 and tuple(gb.shape) == sh2
            scale = max(np.abs(wa).max(), np.abs(wb).max())
            assert np.abs(ga.numpy().ravel() - wa).max() <= 1e-12 * scale
            assert np.abs(gb.numpy().ravel() - wb).max() <= 1e-12 * scale
    with pytest.raises(TypeError):
        helper_diis(torch.zeros(2, dtype=torch.float32), torch.zeros(3), 8)
