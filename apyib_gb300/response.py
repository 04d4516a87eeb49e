"""First-order response of the CISD_SO / CID_SO amplitudes to a perturbation.

For a perturbation x of the integrals (a magnetic-field component or a nuclear
displacement: dF = dF/dx, dERI = d<pq||rs>/dx, orbital response included by the
caller), apyib/analytic_aats.py:757-875 differentiates the amplitude equations
r(t) = c + L t - E t = 0 with E = sum t EW the projected energy:

    r^x = (c^x + L^x t) + L t^x - E^x t - E t^x = 0,
    E^x = sum t EW^x + sum t^x EW,

and solves for t^x by the same Jacobi + DIIS iteration as the amplitudes
(t^x += r^x / D, apyib/utils.py:104-140), starting from the guess of
apyib/analytic_aats.py:738-757.  The residual kernel is linear in the
integrals, so a second plan holding (dF, dERI) gives c^x + L^x t as its residual
at t with the constant terms and no energy term; the first plan gives
L t^x - E t^x.  Everything runs on the GPU through the library's residual,
update, Gram and combination entry points."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .cisd import _DIIS, _lt

_PREC = {"fp64": _lib.PREC_FP64, "ozaki": _lib.PREC_OZAKI, "df64": _lib.PREC_DF64}


def solve_response(plan, plan_x, t, E, params, precision="fp64", print_level=0, history=None):
    """Perturbed amplitudes t^x and the projected-energy derivative E^x.

    plan   -- the converged problem's plan (integrals F, <pq||rs>)
    plan_x -- a plan of the same shape holding the integral derivatives
              (set_fock(dF_SO, eps_so); blocks_from_*(dERI))
    t, E   -- converged packed amplitudes and energy of ``plan``
    params -- e_convergence, d_convergence, max_iterations, DIIS (as the reference)
    precision -- 'fp64' (FP64 pipe), 'ozaki' or 'df64' (FP64-accurate GEMMs off the FP64 pipe)

    Returns (E^x, t^x) with t^x packed like t."""
    return solve_responses(plan, [plan_x], t, E, params, precision=precision, print_level=print_level,
                           histories=None if history is None else [history])[0]


def solve_responses(plan, plan_xs, t, E, params, precision="fp64", print_level=0, histories=None):
    """solve_response for several perturbations of one converged problem, in lockstep:
    each iteration issues every unconverged response's residual, update, DIIS Gram row
    and extrapolation, and two host round trips serve all of them (the Gram rows, then
    the energies and step norms).  Each response follows exactly the iteration, DIIS
    history and convergence test it would follow alone.  Returns [(E^x, t^x), ...]."""
    for px in plan_xs:
        if px.o != plan.o or px.v != plan.v or px.singles != plan.singles:
            raise ValueError("plan_x must have the shape of plan")
    prec = _PREC[precision]
    if prec != _lib.PREC_FP64 and not plan.mixed:
        raise ValueError("FP64-accurate tensor-core / double-float residuals need a mixed plan")
    e_conv, d_conv = params["e_convergence"], params["d_convergence"]
    maxit = params["max_iterations"]
    use_diis = params["DIIS"]
    singles = plan.singles
    K = len(plan_xs)
    if K == 0:
        return []
    dev = t.device
    out = torch.empty((K, 16), dtype=torch.complex128, device=dev)     # (E, s1, s2) per response
    gram = torch.empty((K, 16), dtype=torch.complex128, device=dev)
    norms = torch.empty((K, 2), dtype=torch.float64, device=dev)
    rx = []
    for k, px in enumerate(plan_xs):
        rx.append(px.residual(t, 0.0, prec, flags=_lib.RES_CONST))     # c^x + L^x t
        if prec != _lib.PREC_FP64:
            px.check_status()
        px.combine_into([t], [1.0], t, t, out[k])                       # sum t EW^x
    Ex_t = [complex(x) for x in out[:, 0].cpu().numpy()]
    # guess: one Jacobi step from t^x = 0 with E^x = sum t EW^x
    dt = []
    for k in range(K):
        d = plan.update(torch.zeros_like(t), plan.lincomb([rx[k], t], [1.0, -Ex_t[k]]))
        plan.combine_into([d], [1.0], d, d, out[k])
        dt.append(d)
    dE = [Ex_t[k] + complex(x) for k, x in enumerate(out[:, 0].cpu().numpy())]
    diis = [_DIIS(plan) for _ in range(K)]
    first = [True] * K
    active = list(range(K))
    it = 1
    while it <= maxit and active:
        dE_old = list(dE)
        R, dt_new, unconj = {}, {}, {}
        for k in active:
            rl = plan.residual(dt[k], E, prec, flags=_lib.RES_ETERM)   # L t^x - E t^x
            if prec != _lib.PREC_FP64:
                plan.check_status()
            R[k] = plan.lincomb([rx[k], rl, t], [1.0, 1.0, -dE[k]])
            dt_new[k] = plan.update(dt[k], R[k])
            if use_diis:                     # _DIIS.push, its Gram row left on the device
                h = diis[k]
                if first[k]:
                    plan.dots_into(R[k], [R[k]], gram[k])
                else:
                    while len(h.e) > h.max:
                        h.e.pop(0)
                        h.t.pop(0)
                        h.B = h.B[1:, 1:]
                    plan.dots_into(R[k], h.e + [R[k]], gram[k])
        g = gram.cpu().numpy() if use_diis else None
        for k in active:
            if use_diis:
                h = diis[k]
                if first[k]:
                    h.e, h.t = [R[k]], [dt_new[k]]
                    h.B = np.array([[g[k, 0]]], dtype=np.complex128)
                    first[k] = False
                else:
                    n = len(h.e)
                    Bn = np.zeros((n + 1, n + 1), dtype=np.complex128)
                    Bn[:n, :n] = h.B
                    Bn[:n, n] = g[k, :n]
                    Bn[n, :n] = np.conj(g[k, :n])
                    Bn[n, n] = g[k, n]
                    h.B = Bn
                    h.e.append(R[k])
                    h.t.append(dt_new[k])
                ys, c = h.t, h.coefficients()
            else:
                ys, c = [dt_new[k]], [1.0]
            nxt = plan.vec()
            plan.combine_into(ys, c, dt[k], nxt, out[k])
            # |change| with conjugation, where apyib/analytic_aats.py:868-879 sums the unconjugated
            # squares: the reference solves its magnetic responses in real arithmetic (the factor i
            # taken out), while here a magnetic-field perturbation gives purely imaginary t^x, whose
            # unconjugated sum of squares is negative and would pass the reference's real-part
            # comparison at every iteration (histories keep both forms)
            diff = nxt - dt[k]
            norms[k, 0] = diff[:plan.n1].abs().pow(2).sum()
            norms[k, 1] = diff[plan.n1:].abs().pow(2).sum()
            if histories is not None:       # the reference's unconjugated sums, for the record
                unconj[k] = (diff[:plan.n1].pow(2).sum(), 4.0 * diff[plan.n1:].pow(2).sum())
            dt[k] = nxt
        ev = out[:, 0].cpu().numpy()
        nv = norms.cpu().numpy()
        uc = {k: (complex(a), complex(b)) for k, (a, b) in unconj.items()}
        for k in list(active):
            dE[k] = Ex_t[k] + complex(ev[k])
            rms1 = np.sqrt(float(nv[k, 0]))
            rms2 = np.sqrt(4.0 * float(nv[k, 1]))
            ddE = dE_old[k] - dE[k]
            if histories is not None:
                histories[k].append(dict(iteration=it, dE=dE[k], delta=ddE, rms_t1=complex(rms1),
                                         rms_t2=complex(rms2),
                                         rms_t1_unconj=complex(np.sqrt(np.complex128(uc[k][0]))),
                                         rms_t2_unconj=complex(np.sqrt(np.complex128(uc[k][1])))))
            if print_level > 0:
                print(" %02d %20.12f %20.12f %20.12f %20.12f" % (it, dE[k].real, ddE.real, rms1.real, rms2.real))
            if it > 1 and abs(ddE) < e_conv and _lt(rms2, d_conv) and (not singles or _lt(rms1, d_conv)):
                active.remove(k)
            elif it == maxit:
                print("Not converged.")
        it += 1
    return [(dE[k], dt[k]) for k in range(K)]
