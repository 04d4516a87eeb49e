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
    if plan_x.o != plan.o or plan_x.v != plan.v or plan_x.singles != plan.singles:
        raise ValueError("plan_x must have the shape of plan")
    prec = _PREC[precision]
    if prec != _lib.PREC_FP64 and not plan.mixed:
        raise ValueError("FP64-accurate tensor-core / double-float residuals need a mixed plan")
    e_conv, d_conv = params["e_convergence"], params["d_convergence"]
    maxit = params["max_iterations"]
    singles = plan.singles
    rx = plan_x.residual(t, 0.0, prec, flags=_lib.RES_CONST)     # c^x + L^x t
    if prec != _lib.PREC_FP64:
        plan_x.check_status()
    Ex_t, _, _ = plan_x.combine([t], [1.0], t, t)                 # sum t EW^x
    # guess: one Jacobi step from t^x = 0 with E^x = sum t EW^x
    dt = plan.update(torch.zeros_like(t), plan.lincomb([rx, t], [1.0, -Ex_t]))
    dE_t, _, _ = plan.combine([dt], [1.0], dt, dt)
    dE = Ex_t + dE_t
    diis = _DIIS(plan)
    first = True
    it = 1
    while it <= maxit:
        dE_old = dE
        rl = plan.residual(dt, E, prec, flags=_lib.RES_ETERM)     # L t^x - E t^x
        if prec != _lib.PREC_FP64:
            plan.check_status()
        R = plan.lincomb([rx, rl, t], [1.0, 1.0, -dE])
        dt_new = plan.update(dt, R)
        dt_old = dt.clone()
        if params["DIIS"]:
            diis.push(R, dt_new, first)
            first = False
            c = diis.coefficients()
            dE_t, _, _ = plan.combine(diis.t, c, dt, dt)
        else:
            dE_t, _, _ = plan.combine([dt_new], [1.0], dt, dt)
        dE = Ex_t + dE_t
        # |change| with conjugation: a perturbation such as a magnetic field gives purely
        # imaginary t^x, whose unconjugated sum of squares is negative and would pass the
        # reference's real-part comparison at once
        diff = dt - dt_old
        rms1 = np.sqrt(float(diff[:plan.n1].abs().pow(2).sum().item()))
        rms2 = np.sqrt(4.0 * float(diff[plan.n1:].abs().pow(2).sum().item()))
        ddE = dE_old - dE
        if history is not None:
            history.append(dict(iteration=it, dE=dE, delta=ddE, rms_t1=complex(rms1), rms_t2=complex(rms2)))
        if print_level > 0:
            print(" %02d %20.12f %20.12f %20.12f %20.12f" % (it, dE.real, ddE.real, rms1.real, rms2.real))
        if it > 1 and abs(ddE) < e_conv and _lt(rms2, d_conv) and (not singles or _lt(rms1, d_conv)):
            break
        if it == maxit:
            print("Not converged.")
        it += 1
    return dE, dt
