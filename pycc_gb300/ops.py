"""``torch.ops.gbcc``: the engine's operators registered with PyTorch's dispatcher.

The reference's GPU path dispatches every contraction through torch (``pycc/device.py:64-87``);
these operators put the engine's own FP64 kernels behind the same dispatcher, one operator per
piece of the residual iteration, with the reference's index layouts:

* ``contract(str subscripts, Tensor a, Tensor b) -> Tensor``: ``ContractionBackend.__call__``.
* ``tau(t1, t2, fact1, fact2)``: ``CCwfn.build_tau`` (``pycc/ccwfn.py:432-455``).
* ``fae / fmi / fme / wmnij / wmbej / wmbje / zmbij``: the intermediates
  (``pycc/ccwfn.py:458-715``), ``r_t1 / r_t2`` (``:718-945``) and ``residuals`` (``:321-372``).
  The integrals are passed as the resident blocks: ``ERI`` is the list of the eleven
  <pq|rs> blocks in ``pycc_gb300.hamiltonian.ERI_BLOCKS`` order, ``L`` the five
  L = 2<pq|rs> - <pq|sr> blocks in ``L_BLOCKS`` order; ``F`` is the nmo x nmo Fock matrix.
* ``energy(F, L_oovv, t1, t2)``: ``cc_energy`` (``:1122-1162``).
* ``update_amps_(t1, t2, r1, r2, eps) -> rms``: the Jacobi update of ``solve_cc``
  (``:281-284``), in place, returning the update norm.
* ``diis_dots(x, ys)``, ``lincomb(xs, coef)``: the overlaps and the extrapolation of
  ``helper_diis`` (``pycc/utils.py:330-355``).
* ``t_energy(F, ERI, t1, t2) -> float``: the (T) energy (``pycc/cctriples.py:177-308``).

The operators are registered for the CUDA dispatch key only: called with CPU tensors they raise
NotImplementedError (there is no CPU fallback).  A failing entry point of the C ABI raises
``pycc_gb300.EngineError`` (a RuntimeError) with the library's message.  Tensors are FP64.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .hamiltonian import ERI_BLOCKS, L_BLOCKS, BlockTensor

_DEFS = (
    "contract(str subscripts, Tensor a, Tensor b) -> Tensor",
    "tau(Tensor t1, Tensor t2, float fact1=1.0, float fact2=1.0) -> Tensor",
    "fae(Tensor F, Tensor[] L, Tensor t1, Tensor t2) -> Tensor",
    "fmi(Tensor F, Tensor[] L, Tensor t1, Tensor t2) -> Tensor",
    "fme(Tensor F, Tensor[] L, Tensor t1) -> Tensor",
    "wmnij(Tensor[] ERI, Tensor t1, Tensor t2) -> Tensor",
    "wmbej(Tensor[] ERI, Tensor[] L, Tensor t1, Tensor t2) -> Tensor",
    "wmbje(Tensor[] ERI, Tensor t1, Tensor t2) -> Tensor",
    "zmbij(Tensor[] ERI, Tensor t1, Tensor t2) -> Tensor",
    "r_t1(Tensor F, Tensor[] ERI, Tensor[] L, Tensor t1, Tensor t2, Tensor Fae, Tensor Fme, "
    "Tensor Fmi) -> Tensor",
    "r_t2(Tensor F, Tensor[] ERI, Tensor t1, Tensor t2, Tensor Fae, Tensor Fme, Tensor Fmi, "
    "Tensor Wmnij, Tensor Wmbej, Tensor Wmbje, Tensor Zmbij) -> Tensor",
    "residuals(Tensor F, Tensor[] ERI, Tensor[] L, Tensor t1, Tensor t2) -> (Tensor, Tensor)",
    "energy(Tensor F, Tensor L_oovv, Tensor t1, Tensor t2) -> Tensor",
    "update_amps_(Tensor(a!) t1, Tensor(b!) t2, Tensor r1, Tensor r2, Tensor eps) -> Tensor",
    "diis_dots(Tensor x, Tensor[] ys) -> Tensor",
    "lincomb(Tensor[] xs, float[] coef) -> Tensor",
    "t_energy(Tensor F, Tensor[] ERI, Tensor t1, Tensor t2) -> float",
)

_lib_def = torch.library.Library("gbcc", "DEF")
for _d in _DEFS:
    _lib_def.define(_d)


def _blocks(name, pats, tensors, no, nv):
    if len(tensors) != len(pats):
        raise RuntimeError("gbcc: %s needs its %d blocks (%s), got %d"
                           % (name, len(pats), ", ".join(pats), len(tensors)))
    for pat, t in zip(pats, tensors):
        want = tuple(no if c == "o" else nv for c in pat)
        if tuple(t.shape) != want or t.dtype != torch.float64:
            raise RuntimeError("gbcc: %s block %s must be float64 of shape %s, got %s %s"
                               % (name, pat, want, t.dtype, tuple(t.shape)))
    return BlockTensor(name, no, nv, dict(zip(pats, tensors)))


def _engine(t1, F=None, ERI=None, L=None):
    """An FP64 CCwfn engine over the given blocks: the builders of ``pycc_gb300.CCwfn`` run
    on it unchanged (no amplitude storage, no MP2 guess)."""
    from .ccwfn import CCwfn, WORK_LEN
    from .contract import ContractionBackend
    from .hamiltonian import Hamiltonian
    if t1.dim() != 2:
        raise RuntimeError("gbcc: t1 must be [no, nv]")
    no, nv = t1.shape
    dev = t1.device
    w = CCwfn.__new__(CCwfn)
    w.no, w.nv, w.nmo = no, nv, no + nv
    w.o, w.v = slice(0, no), slice(no, no + nv)
    w.device1, w.stream, w.precision = dev, None, 'DP'
    w._tape, w._mixed = None, None
    w._backend = ContractionBackend(dev, None)
    w.contract = w._contract
    w._work = torch.empty(WORK_LEN, dtype=torch.float64, device=dev)
    eri = _blocks("ERI", ERI_BLOCKS, ERI, no, nv) if ERI is not None else None
    ll = _blocks("L", L_BLOCKS, L, no, nv) if L is not None else None
    if F is not None:
        if tuple(F.shape) != (no + nv, no + nv):
            raise RuntimeError("gbcc: F must be nmo x nmo = %d x %d" % (no + nv, no + nv))
        w.H = Hamiltonian(F, eri, ll, no, nv, dev)
    return w


_impl = torch.library.Library("gbcc", "IMPL", "CUDA")


def _register(name):
    def deco(fn):
        _impl.impl(name, fn)
        return fn
    return deco


@_register("contract")
def _contract(subscripts, a, b):
    from .contract import contract_f64
    return contract_f64(subscripts, a, b)


@_register("tau")
def _tau(t1, t2, fact1=1.0, fact2=1.0):
    return _engine(t1).build_tau(t1.contiguous(), t2.contiguous(), fact1, fact2)


@_register("fae")
def _fae(F, L, t1, t2):
    w = _engine(t1, F, L=L)
    return w.build_Fae(w.o, w.v, F, w.H.L, t1.contiguous(), t2.contiguous())


@_register("fmi")
def _fmi(F, L, t1, t2):
    w = _engine(t1, F, L=L)
    return w.build_Fmi(w.o, w.v, F, w.H.L, t1.contiguous(), t2.contiguous())


@_register("fme")
def _fme(F, L, t1):
    w = _engine(t1, F, L=L)
    return w.build_Fme(w.o, w.v, F, w.H.L, t1.contiguous())


@_register("wmnij")
def _wmnij(ERI, t1, t2):
    w = _engine(t1)
    e = _blocks("ERI", ERI_BLOCKS, ERI, w.no, w.nv)
    return w.build_Wmnij(w.o, w.v, e, t1.contiguous(), t2.contiguous())


@_register("wmbej")
def _wmbej(ERI, L, t1, t2):
    w = _engine(t1)
    e = _blocks("ERI", ERI_BLOCKS, ERI, w.no, w.nv)
    ll = _blocks("L", L_BLOCKS, L, w.no, w.nv)
    return w.build_Wmbej(w.o, w.v, e, ll, t1.contiguous(), t2.contiguous())


@_register("wmbje")
def _wmbje(ERI, t1, t2):
    w = _engine(t1)
    e = _blocks("ERI", ERI_BLOCKS, ERI, w.no, w.nv)
    return w.build_Wmbje(w.o, w.v, e, t1.contiguous(), t2.contiguous())


@_register("zmbij")
def _zmbij(ERI, t1, t2):
    w = _engine(t1)
    e = _blocks("ERI", ERI_BLOCKS, ERI, w.no, w.nv)
    return w.build_Zmbij(w.o, w.v, e, t1.contiguous(), t2.contiguous())


@_register("r_t1")
def _r_t1(F, ERI, L, t1, t2, Fae, Fme, Fmi):
    w = _engine(t1, F, ERI, L)
    return w.r_T1(w.o, w.v, F, w.H.ERI, w.H.L, t1.contiguous(), t2.contiguous(), Fae, Fme, Fmi)


@_register("r_t2")
def _r_t2(F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
    w = _engine(t1, F, ERI)
    return w.r_T2(w.o, w.v, F, w.H.ERI, t1.contiguous(), t2.contiguous(), Fae, Fme, Fmi, Wmnij,
                  Wmbej, Wmbje, Zmbij)


@_register("residuals")
def _residuals(F, ERI, L, t1, t2):
    w = _engine(t1, F, ERI, L)
    return w.residuals(F, t1.contiguous(), t2.contiguous())


@_register("energy")
def _energy(F, L_oovv, t1, t2):
    w = _engine(t1)
    no, nv = w.no, w.nv
    Fov = F[:no, no:]
    out = torch.empty((), dtype=torch.float64, device=t1.device)
    t1c, t2c = t1.contiguous(), t2.contiguous()
    _lib.call("pcg_energy_f64", Fov.data_ptr(), _lib.i64s(Fov.stride()), L_oovv.data_ptr(),
              _lib.i64s(L_oovv.stride()), t1c.data_ptr(), t2c.data_ptr(), no, nv,
              w._work.data_ptr(), w._work.numel(), out.data_ptr(), _lib.stream_handle())
    return out


@_register("update_amps_")
def _update_amps(t1, t2, r1, r2, eps):
    no, nv = t1.shape
    if not (t1.is_contiguous() and t2.is_contiguous()):
        raise RuntimeError("gbcc::update_amps_: t1 and t2 are updated in place and must be "
                           "contiguous")
    if eps.numel() != no + nv:
        raise RuntimeError("gbcc::update_amps_: eps must hold the nmo orbital energies")
    work = torch.empty(4096, dtype=torch.float64, device=t1.device)
    out = torch.empty((), dtype=torch.float64, device=t1.device)
    r1c, r2c, ec = r1.contiguous(), r2.contiguous(), eps.contiguous()
    _lib.call("pcg_update_amps_f64", t1.data_ptr(), t2.data_ptr(), r1c.data_ptr(),
              r2c.data_ptr(), ec.data_ptr(), no, nv, work.data_ptr(), work.numel(),
              out.data_ptr(), _lib.stream_handle())
    return torch.sqrt(out)


@_register("diis_dots")
def _diis_dots(x, ys):
    k = len(ys)
    if not 1 <= k <= 16:
        raise RuntimeError("gbcc::diis_dots: 1 to 16 vectors, got %d" % k)
    xc = x.contiguous()
    yc = [y.contiguous() for y in ys]
    for y in yc:
        if y.numel() != xc.numel():
            raise RuntimeError("gbcc::diis_dots: vectors of different lengths")
    work = torch.empty(1024 * k, dtype=torch.float64, device=x.device)
    out = torch.empty(k, dtype=torch.float64, device=x.device)
    ptrs = (C.c_void_p * k)(*[y.data_ptr() for y in yc])
    _lib.call("pcg_dots_f64", xc.data_ptr(), ptrs, k, xc.numel(), work.data_ptr(), work.numel(),
              out.data_ptr(), _lib.stream_handle())
    return out


@_register("lincomb")
def _lincomb(xs, coef):
    k = len(xs)
    if not 1 <= k <= 16 or len(coef) != k:
        raise RuntimeError("gbcc::lincomb: 1 to 16 vectors with one coefficient each")
    xc = [x.contiguous() for x in xs]
    out = torch.empty_like(xc[0])
    ptrs = (C.c_void_p * k)(*[x.data_ptr() for x in xc])
    cs = (C.c_double * k)(*[float(c) for c in coef])
    _lib.call("pcg_lincomb_f64", ptrs, cs, k, out.numel(), out.data_ptr(), _lib.stream_handle())
    return out


@_register("t_energy")
def _t_energy(F, ERI, t1, t2):
    from .triples import t_energy_fp64
    w = _engine(t1, F, ERI)
    return float(t_energy_fp64(w, t1.contiguous(), t2.contiguous()))


def resident_blocks(H):
    """The ``ERI`` and ``L`` block lists of a :class:`pycc_gb300.Hamiltonian`, in the
    operators' order."""
    return ([H.ERI.blocks[p] for p in ERI_BLOCKS], [H.L.blocks[p] for p in L_BLOCKS])
