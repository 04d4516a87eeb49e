"""Finite-difference AATs in one call (apyib/parallel.py:16-48).

The reference farms the 3N x 3 tensor elements to a process pool.  Here every
element is a handful of GPU contractions (apyib_gb300.aats), so the elements
are evaluated in this process on the current device; ``num_processes`` is
accepted for interface compatibility and not used.
"""
from __future__ import annotations

import numpy as np

from .aats import AAT
from .energy import energy
from .fin_diff import finite_difference
from .hamiltonian import Hamiltonian
from .hf_wfn import hf_wfn


def compute_parallel_aats(parameters, nuc_pert_strength, mag_pert_strength, normalization="full", num_processes=4):
    """(3N, 3) AAT tensor: energy, phase-corrected displaced wavefunctions
    (fin_diff.compute_AAT) and the overlap AATs, spatial or spin-orbital by method."""
    E_list, T_list, C, basis = energy(parameters)
    H = Hamiltonian(parameters)
    wfn = hf_wfn(H)
    fd = finite_difference(parameters, basis, C)
    inputs = fd.compute_AAT(nuc_pert_strength, mag_pert_strength)
    A = AAT(parameters, wfn, C, basis, T_list, *inputs, nuc_pert_strength, mag_pert_strength)
    n3 = 3 * H.molecule.natom()
    I = np.zeros((n3, 3))
    spatial = parameters["method"] in ("RHF", "MP2", "CID", "CISD")
    for a in range(n3):
        for b in range(3):
            I[a, b] = A.compute_spatial_aats(a, b, normalization) if spatial else A.compute_SO_aats(a, b, normalization)
    return I
