"""Small dense complex helpers routed through the library's FP64 GEMM."""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .device import device, ptr, stream_ptr, workspace


def zmm(A, B, transA=False, conjA=False, transB=False, conjB=False, alpha=1.0, out=None, beta=0.0,
        precision=_lib.PREC_FP64):
    """C = alpha * op(A) @ op(B) (+ beta*C) for 2-D complex128 CUDA tensors via agb_zgemm
    (FP64) or agb_cgemm_tf32x3 (complex FP32 as 3xTF32 on the tensor cores)."""
    A = A.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg()
    B = B.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg()
    M, K = (A.shape[1], A.shape[0]) if transA else (A.shape[0], A.shape[1])
    K2, N = (B.shape[1], B.shape[0]) if transB else (B.shape[0], B.shape[1])
    assert K == K2, (A.shape, B.shape, transA, transB)
    sAm, sAk = (A.stride(1), A.stride(0)) if transA else (A.stride(0), A.stride(1))
    sBk, sBn = (B.stride(1), B.stride(0)) if transB else (B.stride(0), B.stride(1))
    if out is None:
        out = torch.empty((M, N), dtype=torch.complex128, device=device())
        beta = 0.0
    alpha, beta = complex(alpha), complex(beta)
    if precision == _lib.PREC_TF32X3 and M > 0 and N > 0 and K > 0:
        nb = _lib.load().agb_cgemm_tf32x3_scratch_bytes(M, N, K)
        buf, sp, _ = workspace(nb)
        buf[:256].zero_()
        _lib.call("agb_cgemm_tf32x3", M, N, K, alpha.real, alpha.imag, ptr(A), sAm, sAk, int(conjA), ptr(B), sBk,
                  sBn, int(conjB), beta.real, beta.imag, ptr(out), out.stride(0), ctypes.c_void_p(sp),
                  ctypes.c_size_t(nb), stream_ptr())
        _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
        del buf
        return out
    nb = _lib.load().agb_zgemm_scratch_bytes(M, N, K) if M > 0 and N > 0 and K > 0 else 0
    if nb:                                    # few output tiles, long K: split K across the SMs
        buf, sp, _ = workspace(nb)
        _lib.call("agb_zgemm_ex", M, N, K, alpha.real, alpha.imag, ptr(A), sAm, sAk, int(conjA), ptr(B), sBk, sBn,
                  int(conjB), beta.real, beta.imag, ptr(out), out.stride(0), ctypes.c_void_p(sp), ctypes.c_size_t(nb),
                  stream_ptr())
        del buf
        return out
    _lib.call("agb_zgemm", M, N, K, alpha.real, alpha.imag, ptr(A), sAm, sAk, int(conjA), ptr(B), sBk, sBn,
              int(conjB), beta.real, beta.imag, ptr(out), out.stride(0), stream_ptr())
    return out


def bmm(A, B, transA=False, conjA=False, transB=False, conjB=False, alpha=1.0):
    """Batched complex product op(A_b) @ op(B_b) for 3-D complex128 CUDA tensors
    [batch, rows, cols] (a batch extent of 1 broadcasts: batch stride 0) through
    agb_zgemm_batched (FP64).  Returns a new [batch, M, N] tensor."""
    A = A.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg()
    B = B.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg()
    if A.dim() == 2:
        A = A.unsqueeze(0)
    if B.dim() == 2:
        B = B.unsqueeze(0)
    nb = max(A.shape[0], B.shape[0])
    if A.shape[0] not in (1, nb) or B.shape[0] not in (1, nb):
        raise ValueError(f"bmm: batch extents {A.shape[0]} and {B.shape[0]} do not broadcast")
    M, K = (A.shape[2], A.shape[1]) if transA else (A.shape[1], A.shape[2])
    K2, N = (B.shape[2], B.shape[1]) if transB else (B.shape[1], B.shape[2])
    assert K == K2, (A.shape, B.shape, transA, transB)
    sAm, sAk = (A.stride(2), A.stride(1)) if transA else (A.stride(1), A.stride(2))
    sBk, sBn = (B.stride(2), B.stride(1)) if transB else (B.stride(1), B.stride(2))
    sAb = A.stride(0) if A.shape[0] == nb and nb > 1 else 0
    sBb = B.stride(0) if B.shape[0] == nb and nb > 1 else 0
    out = torch.empty((nb, M, N), dtype=torch.complex128, device=device())
    a = complex(alpha)
    _lib.call("agb_zgemm_batched", nb, M, N, K, a.real, a.imag, ptr(A), sAm, sAk, sAb, int(conjA), ptr(B), sBk, sBn,
              sBb, int(conjB), 0.0, 0.0, ptr(out), N, M * N, stream_ptr())
    return out


def bdot(X, Y):
    """sum over all but the leading (batch) axis of X * Y (no conjugation), batches
    broadcasting, as batched 1 x K by K x 1 products on the library's GEMM."""
    nb = max(X.shape[0], Y.shape[0])
    Xm = X.reshape(X.shape[0], 1, -1)
    Ym = Y.reshape(Y.shape[0], -1, 1)
    return bmm(Xm, Ym).reshape(nb)


def apply_axis(T, M, axis):
    """out[.., p, ..] = sum_t M[t, p] T[.., t, ..] along ``axis`` of a complex CUDA tensor:
    one library GEMM (agb_zgemm) over the other axes flattened."""
    Tm = T.movedim(axis, -1)
    shp = tuple(Tm.shape)
    out = zmm(Tm.reshape(-1, shp[-1]), M)
    return out.reshape(shp[:-1] + (M.shape[1],)).movedim(-1, axis)


def cg_solve(A, B, tol=1e-14, max_iterations=1000):
    """X with A X = B for a symmetric positive-definite A (n x n) and right-hand sides
    B (n x k), by the conjugate-gradient method with a diagonal (Jacobi) preconditioner,
    every column its own recurrence, products on the library's GEMM; FP64 on the device.
    Stops when every column's residual norm is below tol times its right-hand side's
    norm and raises if that takes more than max_iterations steps.  Used for the
    coupled-perturbed Hartree-Fock equations, whose matrices (the real and imaginary
    orbital Hessians of a stable RHF solution) are positive definite."""
    A = A.to(device=device(), dtype=torch.complex128).contiguous()
    B = B.to(device=device(), dtype=torch.complex128).reshape(A.shape[0], -1).contiguous()
    dinv = (1.0 / torch.diagonal(A).real).to(torch.complex128).reshape(-1, 1)
    X = (dinv * B).contiguous()
    R = B - zmm(A, X)
    Z = dinv * R
    P = Z.clone()
    rz = bdot(R.T.unsqueeze(1).conj(), Z.T.unsqueeze(1)).real
    bn = bdot(B.T.unsqueeze(1).conj(), B.T.unsqueeze(1)).real.sqrt().clamp_min(1e-300)
    for _ in range(max_iterations):
        rn = bdot(R.T.unsqueeze(1).conj(), R.T.unsqueeze(1)).real.sqrt()
        if bool((rn <= tol * bn).all()):
            return X
        AP = zmm(A, P.contiguous())
        pap = bdot(P.T.unsqueeze(1).conj(), AP.T.unsqueeze(1)).real
        alpha = torch.where(pap > 0, rz / pap.clamp_min(1e-300), torch.zeros_like(rz))
        X = X + alpha.to(torch.complex128) * P
        R = R - alpha.to(torch.complex128) * AP
        Z = dinv * R
        rz_new = bdot(R.T.unsqueeze(1).conj(), Z.T.unsqueeze(1)).real
        beta = torch.where(rz > 0, rz_new / rz.clamp_min(1e-300), torch.zeros_like(rz))
        P = Z + beta.to(torch.complex128) * P
        rz = rz_new
    raise RuntimeError("cg_solve: no convergence (is the matrix positive definite?)")


def bdet_inv(S):
    """(det, inverse) of each matrix of a [batch, n, n] complex128 CUDA tensor through
    agb_zdet_inv_batched (FP64 Gauss-Jordan elimination with partial pivoting, n <= 96);
    raises if one is exactly singular."""
    S = S.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
    nb, n, _ = S.shape
    inv = torch.empty_like(S)
    det = torch.empty(nb, dtype=torch.complex128, device=device())
    info = torch.zeros(nb, dtype=torch.int32, device=device())
    _lib.call("agb_zdet_inv_batched", nb, n, ptr(S), n, n * n, ptr(inv), n, n * n, ptr(det), ptr(info),
              stream_ptr())
    if int(info.max().item()) != 0:
        raise ZeroDivisionError("agb_zdet_inv_batched: singular matrix in the batch")
    return det, inv


def last_pair_symmetric(eri):
    """Whether eri[m,n,l,s] == eri[m,n,s,l] exactly, checked once per tensor object and
    version (the verdict rides on the tensor object; one modified in place is checked
    again)."""
    hit = getattr(eri, "_agb_pair_symmetric", None)
    if hit is not None and hit[0] == eri._version:
        return hit[1]
    sym = bool(torch.equal(eri, eri.transpose(2, 3)))
    eri._agb_pair_symmetric = (eri._version, sym)
    return sym


def jk_fock(ERI_AO, D, h, scale, precision="fp64"):
    """F = h + scale * sum_ls D_ls (2 (mn|ls) - (ml|ns)) (apyib/hf_wfn.py:81, apyib/utils.py:249).
    ERIs symmetric in (l, s) (every real AO integral tensor) take a kernel that reads the
    l <= s half: in FP64 (precision 'fp64', the reference's arithmetic) or in double-float
    on the FP32 pipe ('df64', ~1e-14 relative).  Any other tensor takes the general
    double-float kernel."""
    n = D.shape[0]
    eri = ERI_AO.to(device=device(), dtype=torch.float64).contiguous()
    D = D.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
    h = h.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
    F = torch.empty((n, n), dtype=torch.complex128, device=device())
    nb = _lib.load().agb_jk_fock_scratch_bytes(n)
    buf, sp, _ = workspace(nb)
    if precision not in ("fp64", "df64"):
        raise ValueError(f"jk_fock precision must be 'fp64' or 'df64', not {precision!r}")
    if last_pair_symmetric(eri):
        fn = "agb_jk_fock_sym64" if precision == "fp64" else "agb_jk_fock_sym"
    else:
        fn = "agb_jk_fock"
    _lib.call(fn, ptr(eri), n, ptr(D), ptr(h), float(scale), ptr(F), ctypes.c_void_p(sp), ctypes.c_size_t(nb),
              stream_ptr())
    return F
