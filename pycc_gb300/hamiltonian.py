"""GPU-resident MO Hamiltonian: Fock matrix, orbital energies and the o/v blocks of ERI and L.

The reference keeps the full ``nmo^4`` ERI and L on the host and slices them per
contraction (``pycc/hamiltonian.py:57-70``, ``pycc/wavefunction.py:165-169``).  Here only
the blocks the RHF-CCSD residual reads are materialised, once, in HBM; ``ERI[o,v,v,v]``
style indexing with the engine's ``o``/``v`` slices returns the resident block, so the
builders keep the reference's slicing syntax.

Blocks are built either by uploading host arrays (small problems, and every parity test,
so that the reference and the engine consume the same arrays) or on the GPU from the
3-index factor ``B[Q,p,q]`` of a synthetic Hamiltonian: ``<pq|rs> = sum_Q B[Q,p,r] B[Q,q,s]``
through the engine's own FP64 contraction kernel (setup, outside the iteration).
"""
from __future__ import annotations

import types

import numpy as np
import torch

from .contract import contract_f64

# Blocks of <pq|rs> and of L = 2<pq|rs> - <pq|sr> the CCSD residual, energy and MP2 guess read.
ERI_BLOCKS = ("oooo", "ooov", "oovo", "oovv", "ovvo", "ovov", "ovvv", "vvvv", "vvvo", "ovoo",
              "vvoo")
L_BLOCKS = ("oovv", "ovvv", "ooov", "ovvo", "oovo")


class BlockTensor:
    """4-index tensor stored as o/v blocks; ``X[o,v,v,v]`` returns the block."""

    def __init__(self, name, no, nv, blocks):
        self.name = name
        self.no, self.nv = no, nv
        self.o = slice(0, no)
        self.v = slice(no, no + nv)
        self.blocks = dict(blocks)

    def _key(self, s):
        if not isinstance(s, slice):
            raise IndexError("%s: index with the o/v slices only" % self.name)
        if (s.start or 0) == 0 and s.stop == self.no and s.step in (None, 1):
            return "o"
        if s.start == self.no and s.stop == self.no + self.nv and s.step in (None, 1):
            return "v"
        raise IndexError("%s: slice %r is neither the occupied nor the virtual space" % (self.name, s))

    def __getitem__(self, key):
        if not isinstance(key, tuple) or len(key) != 4:
            raise IndexError("%s: four o/v slices expected" % self.name)
        pat = "".join(self._key(s) for s in key)
        try:
            return self.blocks[pat]
        except KeyError:
            raise KeyError("%s block %s is not resident on the GPU" % (self.name, pat)) from None

    def nbytes(self):
        return sum(t.numel() * t.element_size() for t in self.blocks.values())


def _sl(pat, no, nv):
    return [slice(0, no) if c == "o" else slice(no, no + nv) for c in pat]


def _host(x):
    """A float64 numpy view or copy of a numpy array or torch tensor (any device).  Complex
    input is refused: the resident blocks are real, and a complex Fock matrix (a real-time
    field) is passed to ``CCwfn.residuals`` / ``cc_energy`` directly."""
    if isinstance(x, torch.Tensor):
        if torch.is_complex(x):
            raise TypeError("Hamiltonian: complex integrals are not supported")
        x = x.detach().to("cpu", torch.float64).numpy()
    if np.iscomplexobj(x):
        raise TypeError("Hamiltonian: complex integrals are not supported")
    return np.asarray(x, dtype=np.float64)


class Hamiltonian:
    """``H.F``, ``H.eps``, ``H.ERI``, ``H.L`` of the reference, resident on one GPU."""

    def __init__(self, F, ERI, L, no, nv, device):
        self.F = F
        self.eps = torch.diagonal(F).contiguous()
        self.ERI = ERI
        self.L = L
        self.no, self.nv = no, nv
        self.nmo = no + nv
        self.device = device

    @classmethod
    def from_arrays(cls, F, ERI, no, L=None, device="cuda:0"):
        """Upload the needed blocks of full nmo x nmo / nmo^4 arrays in the reference's layout
        (numpy arrays, or torch tensors on any device, as the reference's CPU and GPU modes
        hold them)."""
        device = torch.device(device)
        F, ERI = _host(F), _host(ERI)
        L = None if L is None else _host(L)
        n = F.shape[0]
        nv = n - no
        eri = {}
        for pat in ERI_BLOCKS:
            s = _sl(pat, no, nv)
            eri[pat] = torch.from_numpy(np.ascontiguousarray(ERI[s[0], s[1], s[2], s[3]])).to(device)
        ll = {}
        for pat in L_BLOCKS:
            s = _sl(pat, no, nv)
            if L is not None:
                blk = np.ascontiguousarray(L[s[0], s[1], s[2], s[3]])
            else:
                blk = 2.0 * ERI[s[0], s[1], s[2], s[3]] - ERI[s[0], s[1], s[3], s[2]].swapaxes(2, 3)
            ll[pat] = torch.from_numpy(np.ascontiguousarray(blk)).to(device)
        Ft = torch.from_numpy(F.copy()).to(device)
        return cls(Ft, BlockTensor("ERI", no, nv, eri), BlockTensor("L", no, nv, ll), no, nv, device)

    @classmethod
    def from_full(cls, F, ERI, no):
        """Blocks of a full GPU-resident <pq|rs> (torch, FP64); L formed from it."""
        device = ERI.device
        n = F.shape[0]
        nv = n - no
        eri, ll = {}, {}
        for pat in ERI_BLOCKS:
            s = _sl(pat, no, nv)
            eri[pat] = ERI[s[0], s[1], s[2], s[3]].contiguous()
        for pat in L_BLOCKS:
            s = _sl(pat, no, nv)
            ll[pat] = (2.0 * ERI[s[0], s[1], s[2], s[3]]
                       - ERI[s[0], s[1], s[3], s[2]].transpose(2, 3)).contiguous()
        return cls(F.contiguous().clone(), BlockTensor("ERI", no, nv, eri),
                   BlockTensor("L", no, nv, ll), no, nv, device)

    @classmethod
    def from_factors(cls, fac, device="cuda:0", eri_blocks=ERI_BLOCKS, l_blocks=L_BLOCKS):
        """Build the blocks on the GPU from a :class:`pycc_gb300.synth.SyntheticFactors`."""
        device = torch.device(device)
        no, nv = fac.no, fac.nv
        B = torch.from_numpy(fac.B).to(device)
        Bs = {"o": slice(0, no), "v": slice(no, no + nv)}

        def eri_block(pat, out=None, alpha=1.0, beta=0.0):
            # <pq|rs> = sum_Q B[Q,p,r] B[Q,q,s]
            p, q, r, s = (Bs[c] for c in pat)
            return contract_f64("Qpr,Qqs->pqrs", B[:, p, r], B[:, q, s], out=out, alpha=alpha,
                                beta=beta)

        eri = {pat: eri_block(pat) for pat in eri_blocks}
        ll = {}
        for pat in l_blocks:
            out = eri_block(pat, alpha=2.0)
            p, q, r, s = (Bs[c] for c in pat)
            # - <pq|sr> = - sum_Q B[Q,p,s] B[Q,q,r]
            contract_f64("Qps,Qqr->pqrs", B[:, p, s], B[:, q, r], out=out, alpha=-1.0, beta=1.0)
            ll[pat] = out
        del B
        Ft = torch.from_numpy(fac.F.copy()).to(device)
        return cls(Ft, BlockTensor("ERI", no, nv, eri), BlockTensor("L", no, nv, ll), no, nv, device)

    @classmethod
    def from_npz(cls, path, device="cuda:0"):
        """A Hamiltonian from an ``.npz`` file, without psi4.  Keys: ``no`` (occupied
        orbitals), ``F`` (nmo x nmo Fock matrix), and either ``ERI`` (nmo^4, <pq|rs> order as
        the reference holds it; optionally ``L``) or ``B`` (naux x nmo x nmo, a three-index
        factor with <pq|rs> = sum_Q B[Q,p,r] B[Q,q,s], built into blocks on the GPU)."""
        with np.load(path, allow_pickle=False) as d:
            keys = set(d.files)
            if not {"no", "F"} <= keys or not ({"ERI", "B"} & keys):
                raise KeyError("%s: needs 'no', 'F' and one of 'ERI' / 'B' (has %s)"
                               % (path, sorted(keys)))
            no = int(d["no"])
            F = np.asarray(d["F"], dtype=np.float64)
            n = F.shape[0]
            if F.shape != (n, n) or not 0 < no < n:
                raise ValueError("%s: F must be square with 0 < no < nmo" % path)
            if "B" in keys:
                B = np.ascontiguousarray(d["B"], dtype=np.float64)
                if B.ndim != 3 or B.shape[1:] != (n, n):
                    raise ValueError("%s: B must be naux x nmo x nmo" % path)
                fac = types.SimpleNamespace(no=no, nv=n - no, B=B, F=F)
                return cls.from_factors(fac, device=device)
            ERI = d["ERI"]
            if ERI.shape != (n,) * 4:
                raise ValueError("%s: ERI must be nmo^4" % path)
            L = d["L"] if "L" in keys else None
            return cls.from_arrays(F, ERI, no, L=L, device=device)

    def nbytes(self):
        return self.ERI.nbytes() + self.L.nbytes()
