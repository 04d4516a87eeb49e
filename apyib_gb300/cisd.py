"""Device-resident spin-orbital CISD / CID / MP2 engine.

``CISDPlan`` owns the library plan (antisymmetrised integral blocks, Fock
blocks and per-iteration buffers in one caller-allocated device workspace);
``solve`` runs the Jacobi + DIIS iteration of apyib/ci_wfn.py:263-378
(CISD_SO) or :171-259 (CID_SO) on packed amplitude vectors
t = [t1 (o*v) | t2p (o(o-1)/2 * v(v-1)/2)] held in HBM.

Precision modes:
  * ``fp64``  - every contraction in FP64 (the parity mode);
  * ``mixed`` - residuals as complex FP32 with 3xTF32 tensor-core products
    until the energy change reaches ``switch_tol``, then one high-precision
    residual at a base point t_b and further iterations whose residual is
    r(t) = r64(t_b) + L32(t - t_b) - E_b (t - t_b) - (E - E_b) t,
    i.e. only the small amplitude change goes through the FP32 tensor cores
    (defect correction).  DIIS, the update and all sums stay FP64.  The base
    residual's large GEMMs run on the bf16 tensor cores with six-slice Ozaki
    splitting (``base_precision='ozaki'``, ~1e-12 of sum |a||b|), its small
    ones in double-float; ``'df64'`` runs every GEMM in double-float on the
    FP32 pipe (~2^-44 relative) and ``'fp64'`` on the FP64 pipe; the
    elementwise work is FP64 in every mode.
"""
from __future__ import annotations

import ctypes
import os
import time

import numpy as np
import torch

from . import _lib
from .device import device, empty, ptr, require_cuda, stream_ptr, workspace

_vp = ctypes.c_void_p


class CISDPlan:
    def __init__(self, o, v, singles=True, mixed=False, mp2_only=False):
        require_cuda()
        self.o, self.v = int(o), int(v)
        flags = 0
        if mixed:
            flags |= _lib.PLAN_MIXED
        if not singles:
            flags |= _lib.PLAN_NO_SINGLES
        if mp2_only:
            flags |= _lib.PLAN_MP2
        self.singles = singles and not mp2_only
        self.mixed = mixed
        h = _vp()
        _lib.call("agb_cisd_plan_create", self.o, self.v, flags, ctypes.byref(h))
        self._h = h
        nb = ctypes.c_size_t()
        _lib.call("agb_cisd_plan_workspace_bytes", h, ctypes.byref(nb))
        self.ws_bytes = nb.value
        self._ws_buf, wptr, _ = workspace(nb.value)
        _lib.call("agb_cisd_plan_set_workspace", h, _vp(wptr), ctypes.c_size_t(nb.value))
        n1, n2 = ctypes.c_int64(), ctypes.c_int64()
        _lib.call("agb_cisd_plan_sizes", h, ctypes.byref(n1), ctypes.byref(n2))
        self.n1, self.n2 = n1.value, n2.value
        self.n = self.n1 + self.n2
        pb = _lib.load().agb_vec_partials_bytes(16)
        self._partials = torch.empty(int(pb) // 16 + 16, dtype=torch.complex128, device=device())
        self._out3 = torch.empty(16, dtype=torch.complex128, device=device())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().agb_cisd_plan_destroy(h)
            except Exception:
                pass
            self._h = _vp()

    # ------------------------------------------------------------ set-up
    def set_fock(self, F_SO, eps_so):
        F = F_SO.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        e = torch.as_tensor(eps_so, dtype=torch.float64).to(device()).contiguous()
        self._F, self._eps = F, e
        _lib.call("agb_cisd_set_fock", self._h, ptr(F), ptr(e), stream_ptr())

    def blocks_from_mo(self, ERI_MO):
        g = ERI_MO.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        _lib.call("agb_cisd_blocks_from_mo", self._h, ptr(g), stream_ptr())

    def blocks_from_so(self, ERI_SO):
        g = ERI_SO.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        _lib.call("agb_cisd_blocks_from_so", self._h, ptr(g), stream_ptr())

    def blocks_from_factors(self, B, precision=_lib.PREC_FP64):
        """Blocks from Hermitian factors; precision PREC_FP64, PREC_DF64 (double-float
        products, ~1e-13 relative, several times faster on GB300) or PREC_OZAKI (the
        large products on the bf16 tensor cores, ~1e-12 of sum |a||b|)."""
        Bd = B.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        naux = Bd.shape[0]
        nb = _lib.load().agb_cisd_factor_scratch_bytes(self._h, naux)
        buf, sptr, _ = workspace(nb)
        _lib.call("agb_cisd_blocks_from_factors", self._h, ptr(Bd), ctypes.c_int64(naux), _vp(sptr),
                  ctypes.c_size_t(nb), int(precision), stream_ptr())
        self.check_status()
        del buf

    # ------------------------------------------------------------ kernels
    def vec(self):
        return empty(self.n)

    def guess(self):
        t = self.vec()
        _lib.call("agb_cisd_guess", self._h, ptr(t), stream_ptr())
        return t

    def residual(self, t, E, precision=_lib.PREC_FP64, flags=_lib.RES_CONST | _lib.RES_ETERM, out=None):
        r = self.vec() if out is None else out
        E = complex(E)
        _lib.call("agb_cisd_residual", self._h, int(precision), ptr(t), E.real, E.imag, int(flags), ptr(r),
                  stream_ptr())
        return r

    def check_status(self):
        _lib.call("agb_cisd_status", self._h, stream_ptr())

    def update(self, t, r, out=None):
        o = self.vec() if out is None else out
        _lib.call("agb_cisd_update", self._h, ptr(t), ptr(r), ptr(o), stream_ptr())
        return o

    def dots_into(self, x, ys, out):
        """conj(y_j) . x (weights 1 and 4 on the singles and packed doubles) into the
        device tensor out[:len(ys)], without a host round trip."""
        n = len(ys)
        if n > 16 or out.numel() < n:
            raise ValueError("dots: at most 16 vectors and an output of at least len(ys)")
        arr = (_vp * n)(*[y.data_ptr() for y in ys])
        _lib.call("agb_vec_dots", ctypes.c_int64(self.n1), ctypes.c_int64(self.n2), 1.0, 4.0, ptr(x), arr, n,
                  ptr(out), ptr(self._partials), ctypes.c_size_t(self._partials.numel() * 16), stream_ptr())
        return out

    def dots(self, x, ys):
        return self.dots_into(x, ys, self._out3[:len(ys)]).cpu().numpy().copy()

    def combine_into(self, ys, coefs, t_old, t_new, out3):
        """t_new = sum c_j y_j with (E, s1, s2) left in the device tensor out3[:3]."""
        n = len(ys)
        arr = (_vp * n)(*[y.data_ptr() for y in ys])
        c = np.zeros(2 * n)
        cc = np.asarray(coefs, dtype=np.complex128)
        c[0::2], c[1::2] = cc.real, cc.imag
        carr = (ctypes.c_double * (2 * n))(*c.tolist())
        _lib.call("agb_cisd_combine", self._h, arr, carr, n, ptr(t_old), ptr(t_new), ptr(out3),
                  ptr(self._partials), ctypes.c_size_t(self._partials.numel() * 16), stream_ptr())
        return out3

    def combine(self, ys, coefs, t_old, t_new):
        """t_new = sum c_j y_j; returns (E, s1, s2) as complex numbers."""
        h = self.combine_into(ys, coefs, t_old, t_new, self._out3)[:3].cpu().numpy()
        return complex(h[0]), complex(h[1]), complex(h[2])

    def lincomb(self, ys, coefs, out=None):
        """sum c_j y_j (no host round trip)."""
        o = self.vec() if out is None else out
        self.combine_into(ys, coefs, o if out is not None else ys[0], o, self._out3)
        return o

    def unpack(self, t):
        t1 = torch.empty((self.o, self.v), dtype=torch.complex128, device=device()) if self.singles else None
        t2 = torch.empty((self.o, self.o, self.v, self.v), dtype=torch.complex128, device=device())
        _lib.call("agb_cisd_unpack", self._h, ptr(t), ptr(t1), ptr(t2), stream_ptr())
        return t1, t2

    def pack(self, t1, t2):
        t = self.vec()
        t2 = t2.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        t1 = None if t1 is None else t1.to(device=device(), dtype=torch.complex128).resolve_conj().resolve_neg().contiguous()
        _lib.call("agb_cisd_pack", self._h, ptr(t1), ptr(t2), ptr(t), stream_ptr())
        return t

    def mp2_into(self, t, out):
        """MP2_SO amplitudes into t and the energy into the device tensor out[0]."""
        _lib.call("agb_mp2_so", self._h, ptr(t), ptr(out), ptr(self._partials),
                  ctypes.c_size_t(self._partials.numel() * 16), stream_ptr())
        return t

    def mp2(self):
        t = self.mp2_into(self.vec(), self._out3)
        return complex(self._out3[0].cpu().numpy()), t


def _lt(z, x):
    """numpy's complex < real comparison (lexicographic on (real, imag))."""
    return bool(np.complex128(z) < x)


def _bordered_diis(B):
    """apyib/utils.py:121-135 for a Gram matrix B (n x n complex)."""
    n = B.shape[0]
    Bb = np.zeros((n + 1, n + 1), dtype=np.complex128)
    Bb[:n, :n] = B
    Bb[-1, :] = -1
    Bb[:, -1] = -1
    Bb[-1, -1] = 0
    A = np.zeros(n + 1)
    A[-1] = -1
    return np.linalg.solve(Bb, A)[:-1]


class _DIIS:
    """Device history of error/amplitude vectors with an incrementally built
    Gram matrix; the truncate-then-append order of apyib/utils.py:109-119."""

    def __init__(self, plan, max_diis=7):
        self.plan = plan
        self.max = max_diis
        self.e, self.t = [], []
        self.B = np.zeros((0, 0), dtype=np.complex128)

    def push(self, r, t_new, first):
        if first:
            self.e, self.t = [r], [t_new]
            d = self.plan.dots(r, [r])
            self.B = np.array([[d[0]]], dtype=np.complex128)
            return
        while len(self.e) > self.max:
            self.e.pop(0)
            self.t.pop(0)
            self.B = self.B[1:, 1:]
        d = self.plan.dots(r, self.e + [r])    # conj(e_j) . r
        n = len(self.e)
        Bn = np.zeros((n + 1, n + 1), dtype=np.complex128)
        Bn[:n, :n] = self.B
        Bn[:n, n] = d[:n]
        Bn[n, :n] = np.conj(d[:n])
        Bn[n, n] = d[n]
        self.B = Bn
        self.e.append(r)
        self.t.append(t_new)

    def coefficients(self):
        return _bordered_diis(self.B)


def _save_checkpoint(path, plan, t, E, it):
    tmp = path + ".tmp.npz"
    np.savez(tmp, t=t.cpu().numpy(), E=np.complex128(E), iteration=it, o=plan.o, v=plan.v, n1=plan.n1)
    os.replace(tmp, path)


_BASE_PREC = {"ozaki": _lib.PREC_OZAKI, "df64": _lib.PREC_DF64, "fp64": _lib.PREC_FP64}


def solve(plan, params, precision="fp64", print_level=0, history=None, switch_tol=1e-8, max_mixed=None,
          base_precision="ozaki", checkpoint=None, checkpoint_every=5, resume=False):
    """Jacobi + DIIS CISD_SO (plan.singles) or CID_SO iteration.

    Returns (E, t) with t the packed amplitude vector on the device.  The
    convergence test, DIIS depth and the 'Not converged.' message follow
    apyib/ci_wfn.py:361-378 and apyib/utils.py:104-140.

    checkpoint: path of an .npz file receiving the packed amplitudes, energy and
    iteration every ``checkpoint_every`` iterations (written atomically); with
    resume=True an existing checkpoint of the same shape is the starting point
    (the DIIS history restarts; the reference keeps no checkpoints)."""
    e_conv, d_conv = params["e_convergence"], params["d_convergence"]
    maxit = params["max_iterations"]
    use_diis = params["DIIS"]
    singles = plan.singles
    mixed = precision == "mixed"
    if mixed and not plan.mixed:
        raise ValueError("plan was created without mixed-precision support")
    start_it = 1
    if resume and checkpoint and os.path.exists(checkpoint):
        ck = np.load(checkpoint)
        if int(ck["o"]) != plan.o or int(ck["v"]) != plan.v or int(ck["n1"]) != plan.n1:
            raise ValueError(f"checkpoint {checkpoint} belongs to a different problem")
        t = torch.as_tensor(ck["t"]).to(device())
        start_it = int(ck["iteration"]) + 1
    else:
        t = plan.guess()
    E, _, _ = plan.combine([t], [1.0], t, t)
    diis = _DIIS(plan)
    phase = "tf32" if mixed else "fp64"
    base = None            # (t_b, E_b, r_b) for the defect-correction phase
    first = True
    stats = dict(fp64_residuals=0, tf32_residuals=0)
    it = start_it
    dE_prev = None
    while it <= maxit:
        E_old = E
        t0 = time.perf_counter()
        if phase == "fp64":
            r = plan.residual(t, E, _lib.PREC_FP64)
            stats["fp64_residuals"] += 1
        elif phase == "tf32":
            r = plan.residual(t, E, _lib.PREC_TF32X3)
            stats["tf32_residuals"] += 1
        else:  # defect correction around the FP64 base point
            t_b, E_b, r_b = base
            dlt = plan.lincomb([t, t_b], [1.0, -1.0])
            rl = plan.residual(dlt, 0.0, _lib.PREC_TF32X3, flags=0)
            stats["tf32_residuals"] += 1
            r = plan.lincomb([r_b, rl, dlt, t], [1.0, 1.0, -E_b, -(E - E_b)])
            del dlt, rl
        if phase != "fp64":
            plan.check_status()
        t_new = plan.update(t, r)
        if use_diis:
            diis.push(r, t_new, first)
            first = False
            c = diis.coefficients()
            E, s1, s2 = plan.combine(diis.t, c, t, t)
        else:
            E, s1, s2 = plan.combine([t_new], [1.0], t, t)
        rms_t1 = np.sqrt(np.complex128(s1))
        rms_t2 = np.sqrt(np.complex128(s2))
        dE = E_old - E
        if history is not None:
            history.append(dict(iteration=it, E=E, dE=dE, rms_t1=complex(rms_t1), rms_t2=complex(rms_t2),
                                phase=phase, seconds=time.perf_counter() - t0))
        if print_level > 0:
            print(" %02d %20.12f %20.12f %20.12f %20.12f %20.12f %20.12f %s" % (
                it, E.real, E.imag, dE.real, dE.imag, rms_t1.real, rms_t2.real, phase))
        conv = it > 1 and abs(dE) < e_conv and _lt(rms_t2, d_conv) and (not singles or _lt(rms_t1, d_conv))
        if phase == "tf32":
            stalled = dE_prev is not None and abs(dE) > 0.5 * abs(dE_prev) and abs(dE) < 1e-5
            capped = max_mixed is not None and stats["tf32_residuals"] >= max_mixed
            if (it > 1 and abs(dE) < switch_tol) or stalled or capped or conv:
                # switch to defect correction around an FP64 base residual
                t_b = t.clone()
                tb0 = time.perf_counter()
                r_b = plan.residual(t_b, E, _BASE_PREC[base_precision])
                plan.check_status()
                stats["fp64_residuals"] += 1
                stats["base_residual_s"] = time.perf_counter() - tb0
                base = (t_b, E, r_b)
                phase = "refine"
                diis = _DIIS(plan)
                first = True
                dE_prev = None
                it += 1
                continue
            dE_prev = dE
        if checkpoint and (conv or it % checkpoint_every == 0):
            _save_checkpoint(checkpoint, plan, t, E, it)
        if conv:
            break
        if it == maxit:
            if abs(dE) > e_conv or np.complex128(rms_t2) > d_conv:
                print("Not converged.")
        it += 1
    if history is not None:
        history.append(dict(stats))
    return E, t
