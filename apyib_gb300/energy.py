"""Energy drivers: apyib/energy.py:17-150 on the GPU classes.

``energy(parameters)`` builds the Hamiltonian (AO integrals on the GPU),
solves RHF and runs the method named by ``parameters['method']`` (RHF, MP2,
CID, CISD in spatial orbitals; MP2_SO, CID_SO, CISD_SO in spin orbitals),
returning ``(E_list, T_list, C, basis)`` = ([E_SCF, E_corr, E_nuc],
[t0, t1, t2], C, basis set), plus the Hamiltonian with ``return_H=True``.
``phase_corrected_energy`` first aligns the phase of every MO with the
unperturbed one (utils.compute_phase), as the finite-difference drivers need.
"""
from __future__ import annotations

from .ci_wfn import ci_wfn
from .hamiltonian import Hamiltonian
from .hf_wfn import hf_wfn
from .mp2_wfn import mp2_wfn


def energy(parameters, return_H=False, print_level=0):
    return _energy(parameters, return_H, print_level, None)


def phase_corrected_energy(parameters, unperturbed_basis, unperturbed_C, return_H=False, print_level=0):
    """apyib/energy.py:84-150: energy() with the SCF orbitals phase-aligned to
    ``unperturbed_C`` (on ``unperturbed_basis``) before the correlated method;
    returns the aligned C."""
    return _energy(parameters, return_H, print_level, (unperturbed_basis, unperturbed_C))


def _energy(parameters, return_H, print_level, align):
    H = Hamiltonian(parameters)
    wfn = hf_wfn(H)
    E_SCF, C = wfn.solve_SCF(parameters, print_level)
    if align is not None:
        from .utils import compute_phase
        wfn.C = C = compute_phase(wfn.ndocc, wfn.nbf, align[0], align[1], H.basis_set, C)
    basis = H.basis_set
    E_nuc = H.E_nuc
    E, t0, t1, t2 = 0, 1, 0, 0
    method = parameters["method"]
    if method == "MP2":
        E, t2 = mp2_wfn(parameters, wfn).solve_MP2()
    elif method == "CID":
        E, t2 = ci_wfn(parameters, wfn).solve_CID(print_level)
    elif method == "CISD":
        E, t1, t2 = ci_wfn(parameters, wfn).solve_CISD(print_level)
    elif method == "MP2_SO":
        E, t2 = mp2_wfn(parameters, wfn).solve_MP2_SO()
    elif method == "CID_SO":
        E, t2 = ci_wfn(parameters, wfn).solve_CID_SO(print_level)
    elif method == "CISD_SO":
        E, t1, t2 = ci_wfn(parameters, wfn).solve_CISD_SO(print_level)
    elif method != "RHF":
        raise ValueError(f"unknown method {method!r}")
    E_list = [E_SCF, E, E_nuc]
    if parameters.get("P_nuc", None) is not None:
        E_list.append(H.T_nuc)
    T_list = [t0, t1, t2]
    if print_level == 2 or (align is not None and print_level > 0):
        print("Method: ", method)
        print("Electronic Hartree-Fock Energy: ", E_SCF)
        if method != "RHF":
            print("Electronic Post-Hartree-Fock Energy: ", E)
        print("Total Energy: ", sum(E_list))
        print(parameters)
    if return_H:
        return E_list, T_list, C, basis, H
    return E_list, T_list, C, basis
