"""Analytic nuclear gradients of the RHF, MP2_SO, CID_SO and CISD_SO energies (zero
magnetic field; a uniform electric field allowed), and atomic polar tensors from them.
MP2 enters through the densities of its Hylleraas Lagrangian (adjoint.mp2_densities),
which make its energy stationary in the amplitudes as the CI energies are, so the same
skeleton + orbital-response assembly applies.

The finite-difference route (fin_diff.compute_Nuclear_Gradient) needs 2 x 3N
complete calculations; this one needs one: the SCF, the CI solve, its
Hellmann-Feynman densities (adjoint.densities) and the derivative integrals
(integrals.MintsHelper.oei_deriv_all / eri_deriv_all), plus the coupled-perturbed
Hartree-Fock (CPHF) orbital response, as apyib/analytic_aats.py:84-88, 902-992
organises its zero-field (real-orbital) derivatives:

  dE/dR = dE_RHF/dR + dE_corr/dR
  dE_RHF/dR = sum D h^R + sum D (J^R/2 - K^R/4)[D] - sum W S^R + dE_nuc/dR
              (D = 2 C_o C_o^T, W = 2 C_o eps_o C_o^T)
  dE_corr/dR = sum Y (h^R + G^R[C_o C_o^T]) + sum Gamma_AO (mn|ls)^R          (skeleton)
             + sum (dE/dC + dE/dC*) C U^R                                        (orbital response)

with Y, Gamma_AO the correlation densities in the AO basis and dE/dC the
MO-coefficient gradient (adjoint.mo_coefficient_gradient), and U^R the orbital
response: U_ai from the closed-shell CPHF equations
  (eps_a - eps_i) U_ai + sum_bj [4(ai|bj) - (ab|ij) - (aj|ib)] U_bj
      = -(F^R_ai - eps_i S^R_ai - sum_kl S^R_kl [2(ai|kl) - (ak|il)]),
U_pq = -S^R_pq / 2 within the occupied and within the virtual space (the CI
energy is invariant to those rotations when no orbital is frozen) and
U_ia = -S^R_ia - U_ai.  The CPHF equations (n_vir n_occ square, positive definite
for a stable RHF solution) are solved on the device for all 3N perturbations at
once by preconditioned conjugate gradients (linalg.cg_solve); the integrals,
transforms and contractions run on the GPU through the library.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .device import to_dev
from .integrals import MintsHelper
from .linalg import jk_fock, zmm


def _real_orbitals(C):
    """Remove the arbitrary complex phase of each MO (zero field: the orbitals are real
    up to a phase) and return real C."""
    C = np.asarray(C)
    k = np.argmax(np.abs(C), axis=0)
    ph = C[k, np.arange(C.shape[1])]
    Cr = C * (np.abs(ph) / ph)[None, :]
    if np.abs(Cr.imag).max() > 1e-10:
        raise ValueError("analytic gradients need real orbitals (zero field)")
    return Cr.real.copy()


def nuclear_repulsion_deriv1(mol):
    """d E_nuc / dR (natom, 3) (psi4's Molecule.nuclear_repulsion_energy_deriv1)."""
    R, Z = mol.xyz, mol.Z.astype(float)
    g = np.zeros_like(R)
    for a in range(len(Z)):
        for b in range(len(Z)):
            if a != b:
                d = R[a] - R[b]
                g[a] -= Z[a] * Z[b] * d / np.linalg.norm(d) ** 3
    return g


def geometry_integrals(parameters):
    """The field-independent integrals of an analytic gradient at one geometry: the
    zero-field Hamiltonian, the AO dipole integrals and the derivative integrals
    (overlap, core Hamiltonian, dipole, ERI).  A caller that needs gradients at several
    electric fields (the APT) computes them once and passes them to nuclear_gradient."""
    from .hamiltonian import Hamiltonian
    H0 = Hamiltonian(dict(parameters, F_el=[0.0, 0.0, 0.0]))
    m = MintsHelper(H0.basis_set)
    return {"H0": H0, "mints": m, "mu": [x.np for x in m.ao_dipole()],
            "Sd": m.oei_deriv_all(_lib.OEI_OVERLAP),                                   # [natom, 3, n, n]
            "hd": m.oei_deriv_all(_lib.OEI_KINETIC) + m.oei_deriv_all(_lib.OEI_POTENTIAL),
            "dmu": m.oei_deriv_all(_lib.OEI_DIPOLE),                                   # [natom, 3, 3, n, n]
            "Gd": m.eri_deriv_all()}                                                   # [natom, 3, n, n, n, n]


def _field_hamiltonian(H0, mu, F_el):
    """H0 in the uniform electric field F_el, as Hamiltonian(parameters) builds it
    (apyib/hamiltonian.py:58-68): V - sum_a F_a mu_a and E_nuc(-F)."""
    import copy
    H = copy.copy(H0)
    if any(F_el):
        H.mu_el = mu
        V = H0.V
        for a in range(3):
            V = V - F_el[a] * mu[a]
        H.V = V
    H.E_nuc = H0.molecule.nuclear_repulsion_energy([-f for f in F_el])
    return H


def nuclear_gradient(parameters, precision="fp64", return_parts=False, geometry=None):
    """Analytic dE/dR (natom, 3) of parameters['method'] in RHF, MP2_SO, CID_SO, CISD_SO (or
    the spatial MP2 / CID / CISD, the same energies) at zero magnetic field, in the electric
    field parameters['F_el'] (real orbitals).  ``geometry``: geometry_integrals() of the
    same geometry and basis, to reuse across fields."""
    from .adjoint import mo_coefficient_gradient
    from .hf_wfn import hf_wfn

    method = parameters["method"]
    if method not in ("RHF", "MP2", "MP2_SO", "CID", "CISD", "CID_SO", "CISD_SO"):
        raise ValueError(f"analytic gradients exist for RHF, MP2, CID and CISD, not {method}")
    if any(f != 0.0 for f in parameters["F_mag"]):
        raise ValueError("analytic gradients are implemented at zero magnetic field (real orbitals)")
    F_el = [float(f) for f in parameters["F_el"]]
    if method != "RHF" and parameters.get("freeze_core"):
        raise ValueError("analytic correlated gradients are implemented without frozen core")
    geo = geometry if geometry is not None else geometry_integrals(parameters)
    H = _field_hamiltonian(geo["H0"], geo["mu"], F_el)
    wfn = hf_wfn(H)
    E_scf, C = wfn.solve_SCF(parameters)
    C = _real_orbitals(C)
    wfn.C = C
    nbf, no = wfn.nbf, wfn.ndocc
    natom = H.molecule.natom()
    eps = np.asarray(wfn.eps).real
    Sd, hd, Gd = geo["Sd"], geo["hd"], geo["Gd"]
    for beta in range(3):                                        # h = T + V - F.mu_el (hamiltonian.py:65-68)
        if F_el[beta]:
            hd = hd - F_el[beta] * geo["dmu"][:, :, beta]
    Cd = to_dev(C, torch.float64)
    Co = Cd[:, :no].contiguous()
    Coz = Co.to(torch.complex128)
    Dh = zmm(Coz, Coz, transB=True).real.contiguous()            # C_o C_o^T
    Wd = 2.0 * zmm(Coz * torch.as_tensor(eps[:no]).to(Coz)[None, :], Coz, transB=True).real
    Dc = (2.0 * Dh).to(torch.complex128)
    zero = torch.zeros((nbf, nbf), dtype=torch.complex128, device=Co.device)
    g_hf = np.zeros((natom, 3))
    GR = {}
    for K in range(natom):
        for c in range(3):
            GR[K, c] = Gd[K, c].contiguous()
            two_e = jk_fock(GR[K, c], Dc, zero, 0.25).real
            g_hf[K, c] = float(torch.sum(2.0 * Dh * hd[K, c]) + torch.sum(2.0 * Dh * two_e) - torch.sum(Wd * Sd[K, c]))
    g_hf += nuclear_repulsion_deriv1(H.molecule)
    # E_nuc(F) = E_nuc + (-F) . sum_A Z_A R_A (apyib/hamiltonian.py:58-61)
    g_hf -= np.outer(H.molecule.Z.astype(float), np.asarray(F_el))
    if method == "RHF":
        return (g_hf, {"E": complex(E_scf) + H.E_nuc}) if return_parts else g_hf

    params = dict(parameters, method=method if method.endswith("_SO") else method + "_SO")
    h_AO = torch.as_tensor(np.asarray(H.T) + np.asarray(H.V)).to(Co.device).to(torch.complex128)
    E_corr, dEdC, dEdCc, inter = mo_coefficient_gradient(h_AO, wfn, params, precision=precision,
                                                         return_intermediates=True)
    Y, G_AO = inter["Y"], inter["G_AO"]
    dEdC_r = (dEdC + dEdCc).real                                 # real orbitals, real responses
    # CPHF with all-MO integrals (real orbitals: real integrals), on the device
    from .analytic_aats import _mo
    from .linalg import cg_solve
    from .utils import compute_ERI_MO
    ERI = compute_ERI_MO(params, wfn, [slice(0, 0), slice(0, no), slice(no, nbf), slice(0, nbf)],
                         return_torch=True).real.to(torch.complex128)
    o, v = slice(0, no), slice(no, nbf)
    nv = nbf - no
    e = torch.as_tensor(eps).to(Co.device)
    # A[a,i,b,j] = 4(ai|bj) - (ab|ij) - (aj|ib) + (e_a - e_i) delta
    A = (4.0 * ERI[v, o, v, o] - ERI[v, v, o, o].permute(0, 2, 1, 3) - ERI[v, o, o, v].permute(0, 2, 3, 1))
    A = A.reshape(nv * no, nv * no) + torch.diag((e[no:, None] - e[None, :no]).reshape(-1).to(torch.complex128))
    Gvooo = (2.0 * ERI[v, o, o, o] - ERI[v, o, o, o].permute(0, 2, 1, 3)).reshape(nv * no, no * no)
    Cz = Cd.to(torch.complex128)
    rhs, S_mo = [], {}
    skel = np.zeros((natom, 3))
    for K in range(natom):
        for c in range(3):
            dF_AO = hd[K, c].to(torch.complex128) + jk_fock(GR[K, c], Dh.to(torch.complex128), zero, 1.0)
            skel[K, c] = float((torch.sum(Y * dF_AO) + torch.sum(G_AO * GR[K, c])).real)
            F_mo = _mo(Cz, dF_AO.real)
            S = _mo(Cz, Sd[K, c])
            S_mo[K, c] = S
            B = F_mo[v, o] - S[v, o] * e[None, :no] - zmm(Gvooo, S[o, o].reshape(-1, 1)).reshape(nv, no)
            rhs.append(-B.reshape(-1))
    Uvo = cg_solve(A, torch.stack(rhs, dim=1))
    orb = np.zeros((natom, 3))
    n = 0
    for K in range(natom):
        for c in range(3):
            S = S_mo[K, c]
            U = -0.5 * S.clone()
            U[v, o] = Uvo[:, n].reshape(nv, no)
            U[o, v] = -S[o, v] - U[v, o].T
            dC = zmm(Cz, U).real
            orb[K, c] = float(torch.sum(dEdC_r * dC))
            n += 1
    g = g_hf + skel + orb
    if return_parts:
        return g, {"hf": g_hf, "skeleton": skel, "orbital": orb, "E_corr": E_corr,
                   "E": complex(E_scf) + H.E_nuc + E_corr}
    return g


def apt(parameters, field_step=5e-4, precision="fp64", richardson=True):
    """Atomic polar tensor P[3N, 3] = d mu_beta / d R = -d^2 E / (dR dF_beta) as central
    differences over the electric field of analytic nuclear gradients (length gauge):
    six gradient evaluations per field step (one SCF + one CI solve each), twice with
    Richardson extrapolation (steps 2h and h), where the reference's finite-difference
    APT (apyib/fin_diff.py:151-265) needs 4 x 3N x 3 energies.  The integrals and
    derivative integrals do not depend on the field and are computed once."""
    geo = geometry_integrals(parameters)

    def central(h):
        cols = []
        for beta in range(3):
            g = []
            for s in (1, -1):
                F = list(parameters["F_el"])
                F[beta] += s * h
                g.append(nuclear_gradient(dict(parameters, F_el=F), precision=precision,
                                          geometry=geo).reshape(-1))
            cols.append(-(g[0] - g[1]) / (2 * h))
        return np.stack(cols, axis=1)
    if not richardson:
        return central(field_step)
    return (4.0 * central(field_step) - central(2.0 * field_step)) / 3.0
