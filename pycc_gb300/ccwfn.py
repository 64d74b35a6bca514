"""GPU RHF-CCSD amplitude engine with the reference's ``CCwfn`` interface.

Drop-in for the residual iteration of CrawfordGroup/pycc's ``CCwfn`` (``pycc/ccwfn.py``):
the same method names, argument orders and return layouts -- ``build_tau``,
``build_Fae/Fmi/Fme``, ``build_Wmnij/Wmbej/Wmbje/Zmbij``, ``r_T1``, ``r_T2``, ``residuals``,
``cc_energy`` and ``solve_cc`` -- executed by the CUDA library ``libpycc_gb300.so``:

* ``precision='DP'``: every pairwise contraction is one launch of the FP64 strided DMMA
  kernel (``pcg_contract_f64``) through ``self.contract``; tau builds, the r2
  symmetrisation, the Jacobi update with its norm and the energy are fused FP64 kernels.
* ``precision='MIXED'``: the residual runs on the tcgen05 tensor-core engine
  (``pycc_gb300.mixed``): BF16 operands with FP32 accumulation (FP8 with per-row scales for
  the <ab|ef> ladder), switching to compensated split-BF16x3 products once the update norm
  drops below ``switch_threshold``; amplitudes, denominators, energy, norms and DIIS stay FP64.
* ``precision='SP'``: every contraction in three-piece split-BF16 (six tcgen05 products,
  FP32-class accuracy, the analogue of the reference's float32 mode); FP64 amplitudes.

There is no CPU fallback: ``device='CPU'`` is the reference's own code path.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from .contract import ContractionBackend
from .diis import DIIS
from .exceptions import ConvergenceError, InvalidKeywordError, NumericalError, PyCCError
from .hamiltonian import Hamiltonian

WORK_LEN = 4096


def _lagrange_at_i(nodes):
    """Weights w_k with p(i) = sum_k w_k p(s_k) for every polynomial p of degree < len(nodes)."""
    out = []
    for k, sk in enumerate(nodes):
        num, den = 1.0 + 0.0j, 1.0
        for j, sj in enumerate(nodes):
            if j != k:
                num *= 1j - sj
                den *= sk - sj
        out.append(num / den)
    return tuple(out)


# nodes of the complex-residual evaluation and their weights at s = i
_CNODES = (-2.0, -1.0, 0.0, 1.0, 2.0)
_CWEIGHTS = _lagrange_at_i(_CNODES)


def _ptr(t):
    return t.data_ptr()


def _f64(what, *ts):
    """The FP64 kernels read raw pointers: refuse any other dtype instead of misreading it."""
    for t in ts:
        if t.dtype != torch.float64:
            raise TypeError("%s: float64 tensors expected, got %s" % (what, t.dtype))


def _reference_wfn(w):
    """True for an object shaped like the reference's wave function: an integer ``no`` and an
    ``H`` whose ``F`` and ``ERI`` are full MO arrays (numpy or torch)."""
    H = getattr(w, 'H', None)
    no = getattr(w, 'no', None)
    F, ERI = getattr(H, 'F', None), getattr(H, 'ERI', None)
    return (isinstance(no, (int, np.integer)) and hasattr(F, 'shape') and hasattr(ERI, 'shape')
            and len(F.shape) == 2 and len(ERI.shape) == 4)


class CCwfn:
    """RHF-CCSD wave function on one GPU (mirrors ``pycc/ccwfn.py:32-213``).

    Parameters
    ----------
    scf_wfn : Hamiltonian or object with an ``H`` attribute
        The MO Hamiltonian (see :class:`pycc_gb300.Hamiltonian`); replaces the psi4 SCF
        wave function the reference reads its integrals from.
    model : 'CCSD' or 'CCSD(T)'
    device : 'GPU'
    precision : 'DP', 'SP' or 'MIXED'
    switch_threshold : float
        MIXED only: update norm below which contractions switch to split-BF16x3.
    vvvv_fp8 : bool
        MIXED only: run the <ab|ef> ladder in FP8 before the switch.
    """

    VALID_MODELS = ['CCD', 'CC2', 'CCSD', 'CCSD(T)', 'CC3']
    SUPPORTED_MODELS = ['CCSD', 'CCSD(T)']

    def __init__(self, scf_wfn, **kwargs):
        time_init = time.time()
        model = kwargs.pop('model', 'CCSD').upper()
        if model not in self.VALID_MODELS:
            raise InvalidKeywordError('model', model, self.VALID_MODELS)
        if model not in self.SUPPORTED_MODELS:
            raise NotImplementedError("pycc_gb300 runs the RHF CCSD / CCSD(T) path only (got %r)" % model)
        self.model = model
        device = kwargs.pop('device', 'GPU').upper()
        if device not in ('CPU', 'GPU'):
            raise InvalidKeywordError('device', device, ['CPU', 'GPU'])
        if device == 'CPU':
            raise NotImplementedError("pycc_gb300 is the GPU engine; device='CPU' is the reference's path")
        self.device = device
        precision = kwargs.pop('precision', 'DP').upper()
        if precision not in ('DP', 'SP', 'MIXED'):
            raise InvalidKeywordError('precision', precision, ['DP', 'SP', 'MIXED'])
        self.precision = precision
        self.switch_threshold = float(kwargs.pop('switch_threshold', 1e-5))
        self.vvvv_fp8 = bool(kwargs.pop('vvvv_fp8', True))
        self.quiet = bool(kwargs.pop('quiet', True))
        orbital_basis = kwargs.pop('orbital_basis', 'spatial')
        if orbital_basis != 'spatial':
            raise NotImplementedError("pycc_gb300 runs the closed-shell spatial-orbital path only")
        self.orbital_basis = orbital_basis
        local = kwargs.pop('local', None)
        if local is not None:
            raise NotImplementedError("local correlation is not part of the GPU engine")
        self.local = None
        self._reference_options(kwargs)
        if kwargs:
            raise PyCCError("Unknown keyword argument(s): %s" % ", ".join(sorted(kwargs)))

        H = scf_wfn if isinstance(scf_wfn, Hamiltonian) else getattr(scf_wfn, 'H', None)
        if not isinstance(H, Hamiltonian) and _reference_wfn(scf_wfn):
            # a reference-style wave function (pycc's own CCwfn, for one): its MO Hamiltonian
            # (full F, ERI and L arrays, pycc/hamiltonian.py) and its active occupied count
            dev = getattr(scf_wfn, 'device1', None)
            dev = dev if isinstance(dev, torch.device) else torch.device('cuda:0')
            H = Hamiltonian.from_arrays(H.F, H.ERI, int(scf_wfn.no), L=getattr(H, 'L', None),
                                        device=dev)
        if not isinstance(H, Hamiltonian):
            raise TypeError("CCwfn needs a pycc_gb300.Hamiltonian, an object carrying one as .H, "
                            "or a reference-style wave function (.no and .H with F and ERI)")
        _lib.load()
        self.H = H
        self.no, self.nv, self.nmo = H.no, H.nv, H.nmo
        self.nfzc = 0
        self.eref = float(getattr(scf_wfn, 'eref', 0.0))
        self.o = slice(0, self.no)
        self.v = slice(self.no, self.nmo)
        self.device1 = H.device
        self.stream = None
        self._backend = ContractionBackend(self.device1, self.stream)
        self._tape = None         # set by pycc_gb300.adjoint while a residual is recorded
        self._keep_tape = False   # solve_cc(keep_tape=True): tape every iteration's residual
        self._last_tape = None    # (tape, r1, r2) of the last taped iteration
        self._tape_version = None # amplitude version the kept tape belongs to
        self.contract = self._contract
        self._work = torch.empty(WORK_LEN, dtype=torch.float64, device=self.device1)
        self._scalars = torch.zeros(8, dtype=torch.float64, device=self.device1)

        no, nv = self.no, self.nv
        eps = H.eps
        eps_o, eps_v = eps[:no], eps[no:]
        self.Dijab = (eps_o.reshape(-1, 1, 1, 1) + eps_o.reshape(-1, 1, 1)
                      - eps_v.reshape(-1, 1) - eps_v)
        self.Dia = eps_o.reshape(-1, 1) - eps_v
        # amplitudes live in one flat FP64 vector [t1 | t2] (the DIIS vector)
        self._amps = torch.zeros(no * nv + no * no * nv * nv, dtype=torch.float64,
                                 device=self.device1)
        self.t2.copy_(H.ERI[self.o, self.o, self.v, self.v] / self.Dijab)
        self._mixed = None
        self._warm_start = False  # set by load_amplitudes
        self.ecc = None
        self.niter = 0
        self.timing = {"init": time.time() - time_init}

    def _reference_options(self, kwargs):
        """The reference's other constructor options (``pycc/ccwfn.py:76-160``,
        ``pycc/wavefunction.py:111-160``), validated as it validates them.  Options whose
        default leaves the RHF-CCSD path unchanged are accepted; switching on a feature
        outside that path raises NotImplementedError."""
        if 'frozen_core' in kwargs:
            raise TypeError("the 'frozen_core' argument was removed; the frozen core is taken "
                            "from the SCF reference")
        self.make_t3_density = bool(kwargs.pop('make_t3_density', False))
        for name, what in (('store_triples', "stored CC3 triples"),
                           ('field', "a finite field"),
                           ('localize_occ', "localised occupied orbitals")):
            if kwargs.pop(name, False):
                raise NotImplementedError("%s=True: %s are not part of the GPU engine"
                                          % (name, what))
        self.field_strength = kwargs.pop('field_strength', 0.0)
        self.field_axis = kwargs.pop('field_axis', 'Z')
        self.local_cutoff = kwargs.pop('local_cutoff', 1e-5)
        for name, default, valid in (('it2_opt', True, [True, False]),
                                     ('filter', False, [True, False])):
            val = kwargs.pop(name, default)
            if val not in valid:
                raise InvalidKeywordError(name, val, valid)
            setattr(self, name, val)
        local_mos = str(kwargs.pop('local_mos', 'PIPEK_MEZEY')).upper()
        if local_mos not in ('PIPEK_MEZEY', 'BOYS'):
            raise InvalidKeywordError('local_mos', local_mos, ['PIPEK_MEZEY', 'BOYS'])
        self.local_mos = local_mos
        self.store_triples = self.field = False
        # for CCSD the flag changes nothing (the reference's CC3 triples read it); complex
        # amplitudes are recognised by their dtype
        self.real_time = bool(kwargs.pop('real_time', False))

    # -- amplitude views ------------------------------------------------------------------
    @property
    def t1(self):
        no, nv = self.no, self.nv
        return self._amps[:no * nv].view(no, nv)

    @t1.setter
    def t1(self, value):
        self.t1.copy_(value)

    @property
    def t2(self):
        no, nv = self.no, self.nv
        return self._amps[no * nv:].view(no, no, nv, nv)

    @t2.setter
    def t2(self, value):
        self.t2.copy_(value)

    def _st(self):
        return _lib.stream_handle(self.stream)

    # -- amplitude checkpoint -------------------------------------------------------------
    def save_amplitudes(self, path):
        """Write t1, t2 (FP64) with the sizes and the last converged energy to an ``.npz``
        file, to restart or warm-start ``solve_cc`` later (``load_amplitudes``)."""
        np.savez(path, t1=self.t1.cpu().numpy(), t2=self.t2.cpu().numpy(), no=self.no,
                 nv=self.nv, ecc=np.nan if self.ecc is None else float(self.ecc))

    def load_amplitudes(self, path):
        """Set t1, t2 from a file written by ``save_amplitudes`` (the sizes must match);
        ``solve_cc`` then iterates from them instead of the MP2 guess.  In MIXED / SP the
        next solve starts in the final precision stage: the fast stages' rounding would only
        move converged amplitudes away."""
        with np.load(path, allow_pickle=False) as d:
            if (int(d["no"]), int(d["nv"])) != (self.no, self.nv):
                raise ValueError("%s holds amplitudes for no=%d, nv=%d, not no=%d, nv=%d"
                                 % (path, int(d["no"]), int(d["nv"]), self.no, self.nv))
            self.t1 = torch.from_numpy(np.asarray(d["t1"], dtype=np.float64)).to(self.device1)
            self.t2 = torch.from_numpy(np.asarray(d["t2"], dtype=np.float64)).to(self.device1)
        self._warm_start = True

    def _contract(self, subscripts, *operands, out=None, alpha=1.0, beta=0.0):
        """``self.contract`` (pycc/device.py:64-87) on the FP64 engine; recorded on the
        adjoint tape when one is active."""
        fresh = out is None
        res = self._backend(subscripts, *operands, out=out, alpha=alpha, beta=beta)
        if self._tape is not None:
            self._tape.record("contract", subscripts, operands[0], operands[1], res, alpha,
                              0.0 if fresh else beta)
        return res

    def _copy(self, X):
        """Contiguous copy of a (possibly strided) 2- or 4-index tensor (FP64 kernel)."""
        if X.dim() == 2:
            X4 = X.reshape(1, 1, *X.shape) if X.is_contiguous() else X.unsqueeze(0).unsqueeze(0)
            out = torch.empty(X.shape, dtype=torch.float64, device=X.device)
            self._combine(1.0, X4, 0.0, None, None, out=out.view(1, 1, *X.shape), record=False)
        else:
            out = self._combine(1.0, X, 0.0, None, None, record=False)
        if self._tape is not None:
            self._tape.record("copy", X, out)
        return out

    # -- pycc/ccwfn.py:432-455 ------------------------------------------------------------
    def build_tau(self, t1, t2, fact1=1.0, fact2=1.0):
        """tau_ijab = fact1 t2_ijab + fact2 t_ia t_jb (fused FP64 kernel; complex amplitudes
        through five real evaluations, ``_complex_eval``)."""
        if torch.is_complex(t1) or torch.is_complex(t2):
            return self._complex_eval(lambda a, b: (self.build_tau(a, b, fact1, fact2),),
                                      t1, t2)[0]
        _f64("build_tau", t1, t2)
        if not (t1.is_contiguous() and t2.is_contiguous()):
            raise ValueError("build_tau: t1 and t2 must be contiguous")
        out = torch.empty_like(t2)
        _lib.call("pcg_tau_f64", _ptr(t1), _ptr(t2), self.no, self.nv, float(fact1), float(fact2),
                  _ptr(out), self._st())
        if self._tape is not None:
            self._tape.record("tau", t1, t2, float(fact1), float(fact2), out)
        return out

    def _combine(self, a, X, b, Y, perm_y, out=None, record=True):
        """out_pqrs = a X_pqrs + b Y_perm (4-index; perm_y permutes Y's axes)."""
        _f64("_combine", X, *([Y] if Y is not None else []), *([out] if out is not None else []))
        fresh = out is None
        ext = list(X.shape)
        if out is None:
            out = torch.empty(ext, dtype=torch.float64, device=X.device)
        ys = [0, 0, 0, 0]
        if Y is not None:
            Yp = Y.permute(*perm_y)
            ys = list(Yp.stride())
        _lib.call("pcg_combine4_f64", _lib.i64s(ext), float(a), _ptr(X), _lib.i64s(X.stride()),
                  float(b), _ptr(Y) if Y is not None else None, _lib.i64s(ys), _ptr(out),
                  _lib.i64s(out.stride()), self._st())
        if record and self._tape is not None:
            if not fresh:
                raise ValueError("_combine: only fresh outputs can be recorded")
            self._tape.record("combine", float(a), X, float(b), Y, perm_y, out)
        return out

    # -- pycc/ccwfn.py:458-498 ------------------------------------------------------------
    def build_Fae(self, o, v, F, L, t1, t2):
        c = self.contract
        Fae = self._copy(F[v, v])
        c('me,ma->ae', F[o, v], t1, out=Fae, alpha=-0.5, beta=1.0)
        c('mf,mafe->ae', t1, L[o, v, v, v], out=Fae, beta=1.0)
        c('mnaf,mnef->ae', self.build_tau(t1, t2, 1.0, 0.5), L[o, o, v, v], out=Fae, alpha=-1.0,
          beta=1.0)
        return Fae

    # -- pycc/ccwfn.py:501-534 ------------------------------------------------------------
    def build_Fmi(self, o, v, F, L, t1, t2):
        c = self.contract
        Fmi = self._copy(F[o, o])
        c('ie,me->mi', t1, F[o, v], out=Fmi, alpha=0.5, beta=1.0)
        c('ne,mnie->mi', t1, L[o, o, o, v], out=Fmi, beta=1.0)
        c('inef,mnef->mi', self.build_tau(t1, t2, 1.0, 0.5), L[o, o, v, v], out=Fmi, beta=1.0)
        return Fmi

    # -- pycc/ccwfn.py:537-565 ------------------------------------------------------------
    def build_Fme(self, o, v, F, L, t1):
        Fme = self._copy(F[o, v])
        self.contract('nf,mnef->me', t1, L[o, o, v, v], out=Fme, beta=1.0)
        return Fme

    # -- pycc/ccwfn.py:568-604 ------------------------------------------------------------
    def build_Wmnij(self, o, v, ERI, t1, t2):
        c = self.contract
        W = self._copy(ERI[o, o, o, o])
        c('je,mnie->mnij', t1, ERI[o, o, o, v], out=W, beta=1.0)
        c('ie,mnej->mnij', t1, ERI[o, o, v, o], out=W, beta=1.0)
        c('ijef,mnef->mnij', self.build_tau(t1, t2), ERI[o, o, v, v], out=W, beta=1.0)
        return W

    # -- pycc/ccwfn.py:607-646 ------------------------------------------------------------
    def build_Wmbej(self, o, v, ERI, L, t1, t2):
        c = self.contract
        W = self._copy(ERI[o, v, v, o])
        c('jf,mbef->mbej', t1, ERI[o, v, v, v], out=W, beta=1.0)
        c('nb,mnej->mbej', t1, ERI[o, o, v, o], out=W, alpha=-1.0, beta=1.0)
        c('jnfb,mnef->mbej', self.build_tau(t1, t2, 0.5, 1.0), ERI[o, o, v, v], out=W, alpha=-1.0,
          beta=1.0)
        c('njfb,mnef->mbej', t2, L[o, o, v, v], out=W, alpha=0.5, beta=1.0)
        return W

    # -- pycc/ccwfn.py:649-684 ------------------------------------------------------------
    def build_Wmbje(self, o, v, ERI, t1, t2):
        c = self.contract
        W = self._combine(-1.0, ERI[o, v, o, v], 0.0, None, None)
        c('jf,mbfe->mbje', t1, ERI[o, v, v, v], out=W, alpha=-1.0, beta=1.0)
        c('nb,mnje->mbje', t1, ERI[o, o, o, v], out=W, beta=1.0)
        c('jnfb,mnfe->mbje', self.build_tau(t1, t2, 0.5, 1.0), ERI[o, o, v, v], out=W, beta=1.0)
        return W

    # -- pycc/ccwfn.py:687-715 ------------------------------------------------------------
    def build_Zmbij(self, o, v, ERI, t1, t2):
        return self.contract('mbef,ijef->mbij', ERI[o, v, v, v], self.build_tau(t1, t2))

    # -- pycc/ccwfn.py:718-761 ------------------------------------------------------------
    def r_T1(self, o, v, F, ERI, L, t1, t2, Fae, Fme, Fmi):
        c = self.contract
        r = self._copy(F[v, o].transpose(0, 1))
        c('ie,ae->ia', t1, Fae, out=r, beta=1.0)
        c('mi,ma->ia', Fmi, t1, out=r, alpha=-1.0, beta=1.0)
        t2s = self._combine(2.0, t2, -1.0, t2, (0, 1, 3, 2))
        c('imae,me->ia', t2s, Fme, out=r, beta=1.0)
        c('nf,nafi->ia', t1, L[o, v, v, o], out=r, beta=1.0)
        c('mief,maef->ia', t2s, ERI[o, v, v, v], out=r, beta=1.0)
        c('mnae,nmei->ia', t2, L[o, o, v, o], out=r, alpha=-1.0, beta=1.0)
        return r

    # -- pycc/ccwfn.py:764-791, :886-945 --------------------------------------------------
    def r_T2(self, o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
        r = self._r_T2_half(o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij)
        out = torch.empty_like(r)
        _lib.call("pcg_symmetrize_f64", _ptr(r), self.no, self.nv, _ptr(out), self._st())
        if self._tape is not None:
            self._tape.record("sym", r, out)
        return out

    def _r_T2_half(self, o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij):
        """Half residual of ccwfn.py:922-940.  Two exact refactorings: the Fme dressings
        are folded into the one-body matrices before they multiply t2 (:924-928), and the
        t_ie t_ma <mb|ej> / t_ie t_mb <ma|je> terms (:936-938) are two O(o^3 v^2) steps."""
        c = self.contract
        no, nv = self.no, self.nv
        r = self._combine(0.5, ERI[v, v, o, o].permute(2, 3, 0, 1), 0.0, None, None)
        Fbe = self._copy(Fae)
        c('mb,me->be', t1, Fme, out=Fbe, alpha=-0.5, beta=1.0)
        c('ijae,be->ijab', t2, Fbe, out=r, beta=1.0)
        Fmj = self._copy(Fmi)
        c('je,me->mj', t1, Fme, out=Fmj, alpha=0.5, beta=1.0)
        c('imab,mj->ijab', t2, Fmj, out=r, alpha=-1.0, beta=1.0)
        tau = self.build_tau(t1, t2)
        c('mnab,mnij->ijab', tau, Wmnij, out=r, alpha=0.5, beta=1.0)
        c('ijef,abef->ijab', tau, ERI[v, v, v, v], out=r, alpha=0.5, beta=1.0)
        c('ma,mbij->ijab', t1, Zmbij, out=r, alpha=-1.0, beta=1.0)
        c('imae,mbej->ijab', self._combine(1.0, t2, -1.0, t2, (0, 1, 3, 2)), Wmbej, out=r, beta=1.0)
        c('imae,mbej->ijab', t2, self._combine(1.0, Wmbej, 1.0, Wmbje, (0, 1, 3, 2)), out=r,
          beta=1.0)
        c('mjae,mbie->ijab', t2, Wmbje, out=r, beta=1.0)
        Y = c('ie,mbej->imbj', t1, ERI[o, v, v, o])          # sum_e t_ie <mb|ej>
        c('ma,imbj->ijab', t1, Y, out=r, alpha=-1.0, beta=1.0)
        Y = c('ie,maje->imaj', t1, ERI[o, v, o, v])          # sum_e t_ie <ma|je>
        c('mb,imaj->ijab', t1, Y, out=r, alpha=-1.0, beta=1.0)
        c('ie,abej->ijab', t1, ERI[v, v, v, o], out=r, beta=1.0)
        c('ma,mbij->ijab', t1, ERI[o, v, o, o], out=r, alpha=-1.0, beta=1.0)
        return r

    # -- pycc/ccwfn.py:321-372 ------------------------------------------------------------
    def residuals(self, F, t1, t2, real_time=False):
        """(r1, r2) for the current amplitudes; r2 symmetrised, FP64 on the GPU.

        ``real_time`` is accepted as the reference accepts it: for CCSD it changes nothing
        (only the reference's CC3 triples read it).  Complex F, t1 or t2 -- the amplitudes of
        the reference's real-time propagation -- give complex residuals (``_complex_residuals``).
        """
        if any(torch.is_complex(x) for x in (F, t1, t2)):
            return self._complex_residuals(F, t1, t2)
        if self.precision in ('MIXED', 'SP'):
            return self.mixed_engine().residuals(F, t1, t2)
        o, v = self.o, self.v
        ERI, L = self.H.ERI, self.H.L
        Fae = self.build_Fae(o, v, F, L, t1, t2)
        Fmi = self.build_Fmi(o, v, F, L, t1, t2)
        Fme = self.build_Fme(o, v, F, L, t1)
        Wmnij = self.build_Wmnij(o, v, ERI, t1, t2)
        Wmbej = self.build_Wmbej(o, v, ERI, L, t1, t2)
        Wmbje = self.build_Wmbje(o, v, ERI, t1, t2)
        Zmbij = self.build_Zmbij(o, v, ERI, t1, t2)
        r1 = self.r_T1(o, v, F, ERI, L, t1, t2, Fae, Fme, Fmi)
        r2 = self.r_T2(o, v, F, ERI, t1, t2, Fae, Fme, Fmi, Wmnij, Wmbej, Wmbje, Zmbij)
        return r1, r2

    def _complex_residuals(self, F, t1, t2):
        """Residuals at complex (F, t1, t2) from five real ones (``_complex_eval``): along
        s -> (F_r + s F_i, t_r + s t_i) the residual is a polynomial of degree <= 4 in s
        (terms are at most quartic in t and at most linear in F, and F never multiplies a
        quartic)."""
        return self._complex_eval(lambda *a: self.residuals(*a), F, t1, t2)

    def _complex_eval(self, fn, *args):
        """fn at complex arguments, for an fn whose value along s -> (re + s im) is a
        polynomial of degree <= 4 in s: the Lagrange interpolant through s = -2 .. 2,
        evaluated at s = i, sum_k w_k fn(re + s_k im), exactly.  The weights are at most 2.5
        in modulus, so rounding is not amplified.  fn returns a tuple of real tensors."""
        def parts(x):
            if torch.is_complex(x):
                return x.real.contiguous(), x.imag.contiguous()
            return x.contiguous(), torch.zeros_like(x)
        split = [parts(x) for x in args]
        vals = [fn(*[self._axpy(re, s, im) for re, im in split]) for s in _CNODES]
        out = []
        for q in range(len(vals[0])):
            xs = [v[q] for v in vals]
            re = self._lincomb(xs, [w.real for w in _CWEIGHTS])
            im = self._lincomb(xs, [w.imag for w in _CWEIGHTS])
            out.append(torch.complex(re, im))
        return tuple(out)

    def _axpy(self, x, s, y):
        """x + s y into a fresh contiguous FP64 tensor (FP64 kernel)."""
        _f64("complex evaluation (complex128 / float64 inputs)", x, y)
        out = torch.empty(x.shape, dtype=torch.float64, device=x.device)
        ptrs = (C.c_void_p * 2)(x.data_ptr(), y.data_ptr())
        coef = (C.c_double * 2)(1.0, float(s))
        _lib.call("pcg_lincomb_f64", ptrs, coef, 2, x.numel(), out.data_ptr(), self._st())
        return out

    def _lincomb(self, xs, cs):
        """sum_k cs[k] xs[k] into a fresh tensor (FP64 kernel; the xs are contiguous)."""
        xs = [x.contiguous() for x in xs]
        out = torch.empty_like(xs[0])
        ptrs = (C.c_void_p * len(xs))(*[x.data_ptr() for x in xs])
        coef = (C.c_double * len(xs))(*[float(c) for c in cs])
        _lib.call("pcg_lincomb_f64", ptrs, coef, len(xs), out.numel(), out.data_ptr(), self._st())
        return out

    def t3_density(self):
        """(T) contributions to the densities and the Lambda residuals (``Doo, Dvv, Dov,
        Goovv, Gooov, Gvvvo, S1, S2``), cached as attributes as the reference caches them
        (``pycc/ccwfn.py:1819-1829``); returns the (T) energy.  FP64 on the GPU
        (``pycc_gb300.triples_density``)."""
        from .triples_density import t3_density
        et, dens = t3_density(self)
        for name, value in dens.items():
            setattr(self, name, value)
        return et

    def mixed_engine(self):
        if self._mixed is None:
            from .mixed import MixedResidual
            self._mixed = MixedResidual(self, mode='bf16x6' if self.precision == 'SP' else 'auto')
        return self._mixed

    # -- pycc/ccwfn.py:1122-1162 ----------------------------------------------------------
    def cc_energy_contractions(self, o, v, F, L, t1, t2):
        """The energy as two contractions (the form the adjoint tape records)."""
        E = self.contract('ia,ia->', F[o, v], t1, alpha=2.0)
        self.contract('ijab,ijab->', self.build_tau(t1, t2), L[o, o, v, v], out=E, beta=1.0)
        return E

    def cc_energy(self, o, v, F, L, t1, t2, out=None):
        """E = 2 f_ia t_ia + tau_ijab L_ijab as a 0-d FP64 GPU tensor (fused kernel).  Complex
        F / t1 / t2 (the reference's real-time propagation) give a complex 0-d tensor, through
        five real evaluations (``_complex_eval``)."""
        if any(torch.is_complex(x) for x in (F, t1, t2)):
            return self._complex_eval(lambda f, a, b: (self.cc_energy(o, v, f, L, a, b),),
                                      F, t1, t2)[0]
        _f64("cc_energy", F, t1, t2)
        t1 = t1.contiguous()
        t2 = t2.contiguous()
        Fov = F[o, v]
        Loovv = L[o, o, v, v]
        if out is None:
            out = torch.empty((), dtype=torch.float64, device=t2.device)
        _lib.call("pcg_energy_f64", _ptr(Fov), _lib.i64s(Fov.stride()), _ptr(Loovv),
                  _lib.i64s(Loovv.stride()), _ptr(t1), _ptr(t2), self.no, self.nv,
                  _ptr(self._work), self._work.numel(), _ptr(out), self._st())
        return out

    def update_amplitudes(self, r1, r2):
        """t1 += r1/Dia, t2 += r2/Dijab in place (products with the inverse denominators,
        computed once); returns the two squared partial norms as a 2-element GPU tensor."""
        no, nv = self.no, self.nv
        n1 = no * nv
        if getattr(self, "_inv", None) is None:
            self._inv = torch.empty_like(self._amps)
            _lib.call("pcg_inv_denominators_f64", _ptr(self.H.eps), no, nv, _ptr(self._inv),
                      _ptr(self._inv[n1:]), self._st())
        out = self._scalars[1:3]
        _f64("update_amplitudes", r1, r2)
        r1 = r1.contiguous()
        r2 = r2.contiguous()
        _lib.call("pcg_update_inv_f64", _ptr(self.t1), _ptr(r1), _ptr(self._inv), n1,
                  _ptr(self._work), self._work.numel(), _ptr(out), self._st())
        _lib.call("pcg_update_inv_f64", _ptr(self.t2), _ptr(r2), _ptr(self._inv[n1:]),
                  self._amps.numel() - n1, _ptr(self._work), self._work.numel(),
                  _ptr(out[1:]), self._st())
        return out

    # -- pycc/ccwfn.py:216-319 ------------------------------------------------------------
    def start_iterations(self, max_diis=8):
        """Energy of the current amplitudes and a fresh DIIS history (solve_cc set-up)."""
        o, v, F, L = self.o, self.v, self.H.F, self.H.L
        ecc = float(self.cc_energy(o, v, F, L, self.t1, self.t2))
        self.energies = [ecc]
        self.iter_times = []
        self._last_rms = float('inf')
        # the mixed solver's residual carries ~2^-17 relative rounding: FP32 error vectors
        # hold its updates to better than that, at half the bytes
        edt = torch.float32 if self.precision == 'MIXED' else torch.float64
        if self._warm_start and self.precision != 'DP':
            self.mixed_engine().force_final()
        self._warm_start = False
        return DIIS(self._amps, max_diis, self.stream, error_dtype=edt)

    def iterate(self, diis, niter, start_diis=1, extrapolate=True):
        """One Jacobi + DIIS iteration (ccwfn.py:270-319); returns (ecc, rms).

        The precision schedule of the mixed engine is driven by the previous update norm.
        DIIS bookkeeping runs when ``extrapolate`` is set (solve_cc skips it on the
        iteration that converges, as the reference does).
        """
        t0 = time.time()
        o, v, F, L = self.o, self.v, self.H.F, self.H.L
        if self.precision in ('MIXED', 'SP'):
            self.mixed_engine().select_mode(self._last_rms)
        keep = self._keep_tape and self.precision == 'DP'
        if keep:               # the adjoint can adopt the last iteration's tape
            from .adjoint import Tape
            self._tape = Tape()
        try:
            r1, r2 = self.residuals(F, self.t1, self.t2)
        finally:
            tape, self._tape = self._tape, None
        self._last_tape = (tape, r1, r2) if keep else None
        rms_t = self.update_amplitudes(r1, r2)
        e_t = self.cc_energy(o, v, F, L, self.t1, self.t2)
        del r1, r2
        parts = [e_t.reshape(1), rms_t.reshape(-1)]
        if self.precision in ('MIXED', 'SP'):   # the status words ride on the same read
            parts.append(self.mixed_engine().tc.status.to(torch.float64))
        vals = torch.cat(parts).cpu().numpy()
        ecc, rms = float(vals[0]), math.sqrt(max(float(vals[1] + vals[2]), 0.0))
        if self.precision in ('MIXED', 'SP'):
            self.mixed_engine().tc.check_status(vals[3:])
        self.energies.append(ecc)
        self.iter_times.append(time.time() - t0)
        self.niter = niter
        self._last_rms = rms
        if not (math.isfinite(ecc) and math.isfinite(rms)):
            raise NumericalError("non-finite energy/update norm at iteration %d" % niter)
        return ecc, rms

    def diis_step(self, diis, niter, start_diis=1):
        diis.add_error_vector(self._amps)
        if niter >= start_diis:
            diis.extrapolate(self._amps)       # in place

    def solve_cc(self, e_conv=1e-7, r_conv=1e-7, maxiter=100, max_diis=8, start_diis=1,
                 callback=None, keep_tape=False):
        """Jacobi + DIIS iteration to convergence; returns the correlation energy (float).

        Convergence: |dE| < e_conv and rms < r_conv (ccwfn.py:295).  In the MIXED / SP
        modes the compensated products have a rounding floor; once the final precision
        stage has stopped reducing the update norm for several iterations the energy is
        reported as the mean of the last four iterates (``self.converged_at_floor``).
        Raises :class:`ConvergenceError` if ``maxiter`` is exhausted and
        :class:`NumericalError` if the energy or the update norm turns NaN/Inf.

        ``keep_tape`` (DP): every iteration records its residual on an adjoint tape and the
        last one is kept, so that :class:`pycc_gb300.adjoint.CCSDAdjoint` adopts it instead
        of evaluating the residual again at the converged amplitudes.  The taped residual is
        the converging iteration's, at amplitudes one update (below ``r_conv``) away.
        """
        t_start = time.time()
        self._keep_tape = bool(keep_tape)
        self._tape_version = None
        self.e_conv, self.r_conv, self.maxiter = e_conv, r_conv, maxiter
        self.converged_at_floor = False
        diis = self.start_iterations(max_diis)
        ecc = self.energies[0]
        ediff, rms = -ecc, float('inf')
        if not self.quiet:
            print("iter  %20s  %12s  %12s  %10s  %s" % ("E_corr", "dE", "rms", "time", "precision"))
            print("%4d  %20.15f  %12.3e" % (0, ecc, -ecc))
        for niter in range(1, maxiter + 1):
            ecc_last = ecc
            ecc, rms = self.iterate(diis, niter, start_diis)
            ediff = ecc - ecc_last
            if callback is not None:
                callback(niter, ecc, ediff, rms)
            if not self.quiet:
                stage = self.mixed_engine().mode_name() if self.precision != 'DP' else 'fp64'
                print("%4d  %20.15f  %12.3e  %12.3e  %8.3f s  %s"
                      % (niter, ecc, ediff, rms, self.iter_times[-1], stage))
            done = abs(ediff) < e_conv and rms < r_conv
            if self.precision != 'DP':
                eng = self.mixed_engine()
                if done and not eng.is_final_mode():
                    eng.force_final()          # converged in a fast stage: refine
                    done = False
                elif not done and eng.at_floor() and len(self.energies) > 4:
                    ecc = float(np.mean(self.energies[-4:]))
                    self.converged_at_floor = True
                    self.rms_floor = rms
                    done = True
            if done:
                self.ecc = ecc
                self.timing["solve"] = time.time() - t_start
                self._keep_tape = False
                if self._last_tape is not None:
                    # valid while the amplitudes stay as converged (torch's version counter
                    # of the amplitude buffer records every later in-place change)
                    self._tape_version = self._amps._version
                if self.model == 'CCSD(T)':
                    if self.make_t3_density:
                        et = self.t3_density()
                    else:
                        from .triples import t_energy
                        et = t_energy(self)
                    self.et = et
                    ecc = ecc + et
                    self.ecc = ecc
                return ecc
            self.diis_step(diis, niter, start_diis)
        raise ConvergenceError("CCSD", maxiter, ediff, rms)


ccwfn = CCwfn
