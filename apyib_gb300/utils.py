"""GPU drop-ins for the hot-path helpers of apyib/utils.py.

Same names, arguments and return conventions as the reference; arrays are
returned as NumPy (like the reference) unless ``return_torch=True``.
"""
from __future__ import annotations

import collections
import ctypes
import hashlib

import numpy as np
import torch

from . import _lib
from .device import device, ptr, stream_ptr, to_dev, workspace
from .linalg import jk_fock, zmm


def _ret(t, return_torch):
    return t if return_torch else t.detach().cpu().numpy()


def get_slices(parameters, wfn):
    """apyib/utils.py:184-213."""
    nfzc = wfn.H.basis_set.n_frozen_core()
    nbf = wfn.nbf
    no = wfn.ndocc
    C_list = [slice(0, nfzc), slice(nfzc, no), slice(no, nbf), slice(nfzc, nbf)]
    m = parameters["method"]
    if m in ("RHF", "MP2", "CID", "CISD"):
        I_list = [slice(0, nfzc), slice(0, no - nfzc), slice(no - nfzc, nbf - nfzc), slice(0, nbf - nfzc)]
    elif m in ("MP2_SO", "CID_SO", "CISD_SO"):
        I_list = [slice(0, 2 * nfzc), slice(0, 2 * no - 2 * nfzc), slice(2 * no - 2 * nfzc, 2 * nbf - 2 * nfzc),
                  slice(0, 2 * nbf - 2 * nfzc)]
    else:
        raise ValueError(f"unknown method {m}")
    return C_list, I_list


def compute_F_MO(parameters, wfn, C_list, return_torch=False):
    """apyib/utils.py:217-254: frozen-core operator, J/K Fock build, C^H F C."""
    f, o, v, t = C_list
    C = to_dev(wfn.C)
    h_AO = to_dev(np.asarray(wfn.H.T) + np.asarray(wfn.H.V))
    ERI = to_dev(wfn.H.ERI, torch.float64)
    E_fc = 0
    if parameters["freeze_core"]:
        C_fc = C[:, f]
        D_fc = zmm(C_fc, C_fc, transB=True, conjB=True)
        h_fc = jk_fock(ERI, D_fc, h_AO, 1.0)
        E_fc = complex(torch.sum(D_fc.T * (h_AO + h_fc)).cpu())
        h_AO = h_fc
    Co = C[:, o]
    D = zmm(Co, Co, transB=True, conjB=True)
    F_AO = jk_fock(ERI, D, h_AO, 1.0)
    Ct = C[:, t].contiguous()
    F_MO = zmm(zmm(Ct, F_AO, transA=True, conjA=True), Ct)
    return _ret(F_MO, return_torch), E_fc


_TRANSFORM_PREC = {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI, "df64": _lib.PREC_DF64,
                   "tf32x3": _lib.PREC_TF32X3}


def transform_precision(parameters):
    """Precision of the AO->MO transform for a parameters dict: its 'transform_precision'
    key ('fp64', 'ozaki', 'df64' or 'tf32x3') when present, else Ozaki under
    precision='mixed' (FP64-accurate, ~1e-12 of sum |a||b|, on the tensor cores) and
    FP64 otherwise."""
    key = parameters.get("transform_precision")
    if key is None:
        key = "ozaki" if parameters.get("precision") == "mixed" else "fp64"
    return _TRANSFORM_PREC[key]


def compute_ERI_MO(parameters, wfn, C_list, return_torch=False, precision=None):
    """apyib/utils.py:258-279: four quarter-step AO->MO transform (complex C, real AO ERIs).
    precision: _lib.PREC_FP64, PREC_DF64 (double-float GEMMs on the FP32 pipe, ~1e-13
    relative), PREC_OZAKI (FP64-accurate bf16-slice GEMMs on the tensor cores, ~1e-12 of
    sum |a||b|) or PREC_TF32X3 (tensor cores, ~1e-6 relative); None chooses by
    ``transform_precision(parameters)``."""
    if precision is None:
        precision = transform_precision(parameters)
    t = C_list[3]
    C = to_dev(np.asarray(wfn.C)[:, t])
    ERI = to_dev(wfn.H.ERI, torch.float64)
    nbf, nmo = C.shape
    out = torch.empty((nmo, nmo, nmo, nmo), dtype=torch.complex128, device=device())
    nb = _lib.load().agb_ao2mo_scratch_bytes(nbf, nmo, int(precision))
    buf, sp, _ = workspace(nb)
    _lib.call("agb_ao2mo", ptr(ERI), nbf, ptr(C), nmo, ptr(out), ctypes.c_void_p(sp), ctypes.c_size_t(nb),
              int(precision), stream_ptr())
    torch.cuda.current_stream().synchronize()
    del buf
    return _ret(out, return_torch)


def compute_F_SO(wfn, F_MO, return_torch=False):
    """apyib/utils.py:283-313."""
    F = to_dev(F_MO)
    n = F.shape[0]
    out = torch.empty((2 * n, 2 * n), dtype=torch.complex128, device=device())
    _lib.call("agb_compute_f_so", ptr(F), n, ptr(out), stream_ptr())
    return _ret(out, return_torch)


def compute_ERI_SO(wfn, ERI_MO, return_torch=False):
    """apyib/utils.py:317-365."""
    g = to_dev(ERI_MO)
    n0, n1, n2, n3 = g.shape
    out = torch.empty((2 * n0, 2 * n1, 2 * n2, 2 * n3), dtype=torch.complex128, device=device())
    _lib.call("agb_compute_eri_so", ptr(g), n0, n1, n2, n3, ptr(out), stream_ptr())
    return _ret(out, return_torch)


def solve_general_DIIS(parameters, res_vec, t_vec, e_iter, t_iter, iteration, min_DIIS=1, max_DIIS=7):
    """apyib/utils.py:104-140 on device tensors (e_iter/t_iter: [length, nvec])."""
    res_vec = to_dev(res_vec)
    t_vec = to_dev(t_vec)
    e_iter = to_dev(e_iter)
    t_iter = to_dev(t_iter)
    while e_iter.shape[1] > max_DIIS:
        e_iter = e_iter[:, 1:]
        t_iter = t_iter[:, 1:]
    if iteration != 1:
        e_iter = torch.cat((e_iter, res_vec.reshape(-1, 1)), dim=1)
        t_iter = torch.cat((t_iter, t_vec.reshape(-1, 1)), dim=1)
    e_iter = e_iter.contiguous()
    t_iter = t_iter.contiguous()
    B = zmm(e_iter, e_iter, transA=True, conjA=True).cpu().numpy()
    n = B.shape[0]
    Bb = np.zeros((n + 1, n + 1), dtype=np.complex128)
    Bb[:n, :n] = B
    Bb[-1, :] = -1
    Bb[:, -1] = -1
    Bb[-1, -1] = 0
    A = np.zeros(n + 1)
    A[-1] = -1
    c = np.linalg.solve(Bb, A)[:-1]
    cd = torch.as_tensor(c.reshape(-1, 1)).to(device())
    t_new = zmm(t_iter, cd).reshape(-1)
    return t_new, e_iter, t_iter


_AO_OVERLAPS = collections.OrderedDict()


def _basis_fingerprint(bs):
    """A digest of everything the overlap integrals read from a basis (shell arrays,
    centres, pure/Cartesian), or None for a basis object without them."""
    if not hasattr(bs, "flat"):
        return None
    h = hashlib.sha1(b"pure" if bs.pure else b"cart")
    for k, a in sorted(bs.flat().items()):
        h.update(k.encode())
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _ao_overlap(bra_basis, ket_basis):
    """<bra AO | ket AO> on the device, kept in a small LRU cache keyed by the two bases'
    contents: the finite-difference AAT asks for the overlaps of 25 geometries' MOs
    133 times but for only 19 distinct pairs of geometries (a field moves no nucleus)."""
    from .integrals import MintsHelper
    key = (_basis_fingerprint(bra_basis), _basis_fingerprint(ket_basis))
    if None not in key and key in _AO_OVERLAPS:
        _AO_OVERLAPS.move_to_end(key)
        return _AO_OVERLAPS[key]
    if bra_basis is ket_basis:
        S = MintsHelper(bra_basis).ao_overlap(return_torch=True)
    else:
        S = MintsHelper(bra_basis).ao_overlap(bra_basis, ket_basis, return_torch=True)
    if None not in key:
        _AO_OVERLAPS[key] = S
        while len(_AO_OVERLAPS) > 64:
            _AO_OVERLAPS.popitem(last=False)
    return S


def compute_mo_overlap(ndocc, nbf, bra_basis, bra_wfn, ket_basis, ket_wfn, return_torch=False):
    """apyib/utils.py:370-388: <bra MO p | ket MO q> = C_bra^H S(bra, ket) C_ket, with
    the AO overlap between two bases (two geometries) on the GPU."""
    S = _ao_overlap(bra_basis, ket_basis).to(torch.complex128)
    X = zmm(S, to_dev(ket_wfn))
    out = zmm(to_dev(bra_wfn), X, transA=True, conjA=True)
    return _ret(out, return_torch)


def compute_so_overlap(nbf, mo_overlap, return_torch=False):
    """apyib/utils.py:393-423: spin-orbital overlap, alpha even / beta odd, zero
    between spins (the same spin integration as compute_F_SO)."""
    return compute_F_SO(None, mo_overlap, return_torch)


def compute_phase(ndocc, nbf, unperturbed_basis, unperturbed_wfn, ket_basis, ket_wfn):
    """apyib/utils.py:427-446: divide each ket MO by the phase of its overlap with
    the same unperturbed MO, phase = S_mm / sqrt(S_mm conj(S_mm))."""
    S = compute_mo_overlap(ndocc, nbf, unperturbed_basis, unperturbed_wfn, ket_basis, ket_wfn)
    d = np.diagonal(S)
    N = np.sqrt(d * np.conjugate(d))
    phase = d / N
    return np.asarray(ket_wfn) * (phase ** -1)[None, :]
