"""Restricted Hartree-Fock with a complex Hermitian core Hamiltonian
(drop-in for apyib/hf_wfn.py:9-170).

The nbf^4 J/K Fock build runs on the GPU in one pass over the l <= s half of the
real AO ERIs (agb_jk_fock_sym64: FP64, as the reference's einsum; double-float
agb_jk_fock_sym when parameters['precision'] is 'mixed'); the orthogonaliser X = S^-1/2, the Hermitian diagonalisation,
the DIIS bordered solve and the energy/density sums stay FP64 (NumPy/SciPy on
the host, matrices of size nbf x nbf).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as la
import torch

from .device import to_dev
from .linalg import jk_fock
from .utils import solve_general_DIIS


class hf_wfn(object):
    def __init__(self, H, charge=0):
        self.H = H
        self.nelec = self.nelectron(charge)
        self.ndocc = self.nelec // 2
        self.nbf = H.basis_set.nbf()
        self.C = np.zeros((self.nbf, self.nbf))
        self.eps = np.zeros((self.nbf))
        self.E_SCF = 0

    def nelectron(self, charge):
        nelec = -charge
        for atom in range(self.H.molecule.natom()):
            nelec += self.H.molecule.true_atomic_number(atom)
        return nelec

    def solve_SCF(self, parameters, print_level=0):
        """apyib/hf_wfn.py:36-170; returns (E_SCF, C)."""
        H = self.H
        nbf, nocc = self.nbf, self.ndocc
        H_core = np.asarray(H.T) + np.asarray(H.V)
        S = np.asarray(H.S)
        X = np.linalg.inv(la.sqrtm(S))
        F_p = X @ H_core @ X
        e, C_p = np.linalg.eigh(F_p)
        C = X @ C_p
        D = 2 * C[:, :nocc] @ np.conjugate(C[:, :nocc]).T
        E_SCF = np.sum(0.5 * D * (H_core + H_core))
        E_tot = E_SCF.real + H.E_nuc
        if parameters.get("P_nuc", None) is not None:
            E_tot = E_tot + H.T_nuc
        if print_level > 0:
            print("\n Iter      E_elec(real)       E_elec(imaginary)        E(tot)           Delta_E(real)"
                  "       Delta_E(imaginary)      RMS_D(real)      RMS_D(imaginary)")
            print(" %02d %20.12f %20.12f %20.12f" % (0, E_SCF.real, E_SCF.imag, E_tot))
        ERI = to_dev(H.ERI, torch.float64)
        Hd = to_dev(H_core)
        # FP64 J/K (the reference's arithmetic) unless the caller asked for the mixed path
        jk_precision = "df64" if parameters.get("precision") == "mixed" else "fp64"
        e_iter = F_iter = None
        i = 1
        while i <= parameters["max_iterations"]:
            E_old = E_SCF
            D_old = D
            F = jk_fock(ERI, to_dev(D), Hd, 0.5, precision=jk_precision).cpu().numpy()
            if parameters["DIIS"]:
                SDF = S @ D @ F
                res_vec = np.reshape(X @ (SDF - np.conjugate(SDF.T)) @ X, (-1))
                F_vec = np.reshape(F, (-1))
                if i == 1:
                    F_iter = np.atleast_2d(F_vec).T
                    e_iter = np.atleast_2d(res_vec).T
                F_vec, e_iter, F_iter = solve_general_DIIS(parameters, res_vec, F_vec, e_iter, F_iter, i)
                F = F_vec.cpu().numpy().reshape(nbf, nbf)
            F_p = X @ F @ X
            self.eps, C_p = np.linalg.eigh(F_p)
            C = self.C = X @ C_p
            D = 2 * C[:, :nocc] @ np.conjugate(C[:, :nocc]).T
            E_SCF = np.sum(0.5 * D.T * (H_core + F))
            E_tot = E_SCF + H.E_nuc
            if parameters.get("P_nuc", None) is not None:
                E_tot = E_tot + H.T_nuc
            delta_E = E_SCF - E_old
            rms_D = np.sqrt(np.sum((D_old - D) ** 2))
            if print_level > 0:
                print(" %02d %20.12f %20.12f %20.12f %20.12f %20.12f %20.12f %20.12f" % (
                    i, E_SCF.real, E_SCF.imag, E_tot.real, delta_E.real, delta_E.imag, rms_D.real, rms_D.imag))
            if i > 1:
                if abs(delta_E) < parameters["e_convergence"] and rms_D < parameters["d_convergence"]:
                    break
            if i == parameters["max_iterations"]:
                if abs(delta_E) > parameters["e_convergence"] or rms_D > parameters["d_convergence"]:
                    if print_level > 0:
                        print("Not converged.")
            i += 1
        self.E_SCF = E_SCF
        return E_SCF, self.C
