"""Host logic of the resident Hamiltonian, on CPU: the o/v blocks uploaded from full arrays
(numpy or torch, as the reference's CPU and GPU modes hold them) and L = 2<pq|rs> - <pq|sr>
(pycc/hamiltonian.py:70) formed block by block; BlockTensor indexing with the engine's slices.
"""
import numpy as np
import pytest
import torch

from pycc_gb300.hamiltonian import ERI_BLOCKS, L_BLOCKS, Hamiltonian, _sl


def test_blocks_from_numpy_and_torch(ham_o5v19):
    _, F, ERI, L = ham_o5v19
    no, nv = 5, 19
    Hn = Hamiltonian.from_arrays(F, ERI, no, device="cpu")
    Ht = Hamiltonian.from_arrays(torch.from_numpy(F), torch.from_numpy(ERI), no,
                                 L=torch.from_numpy(L), device="cpu")
    o, v = slice(0, no), slice(no, no + nv)
    assert Hn.ERI[o, v, v, v].is_contiguous()
    for pat in ERI_BLOCKS:
        s = _sl(pat, no, nv)
        want = ERI[s[0], s[1], s[2], s[3]]
        assert np.array_equal(Hn.ERI.blocks[pat].numpy(), want)
        assert np.array_equal(Ht.ERI.blocks[pat].numpy(), want)
    for pat in L_BLOCKS:
        s = _sl(pat, no, nv)
        want = L[s[0], s[1], s[2], s[3]]
        assert np.abs(Hn.L.blocks[pat].numpy() - want).max() < 1e-15      # formed from ERI
        assert np.array_equal(Ht.L.blocks[pat].numpy(), want)              # uploaded as given
    assert np.array_equal(Hn.eps.numpy(), np.diag(F))


def test_block_indexing_errors(ham_o5v19):
    _, F, ERI, _ = ham_o5v19
    H = Hamiltonian.from_arrays(F, ERI, 5, device="cpu")
    o, v = slice(0, 5), slice(5, 24)
    assert H.ERI[v, v, v, v].shape == (19, 19, 19, 19)
    with pytest.raises(KeyError, match="not resident"):
        H.ERI[v, o, o, o]                               # no term of the residual reads vooo
    with pytest.raises(IndexError):
        H.ERI[o, v, v]                                  # three indices
    with pytest.raises(IndexError):
        H.ERI[slice(0, 3), v, v, v]                     # not the occupied space
    with pytest.raises(KeyError, match="not resident"):
        H.L[v, v, v, v]                                 # L keeps only the residual's blocks


def test_complex_input_refused(ham_o5v19):
    _, F, ERI, _ = ham_o5v19
    with pytest.raises(TypeError):
        Hamiltonian.from_arrays(F + 0.01j, ERI, 5, device="cpu")
    with pytest.raises(TypeError):
        Hamiltonian.from_arrays(torch.from_numpy(F).to(torch.complex128), ERI, 5, device="cpu")
