"""CPU restatement of apyib/energy.py:17-81 on the oracle (NumPy) functions.

TEST INFRASTRUCTURE ONLY (the oracle): a geometry string and basis name go
through the oracle integrals (oracle/ints.py), the oracle SCF and the oracle
MP2_SO / CID_SO / CISD_SO solvers (oracle/port.py), with the field terms of
apyib/hamiltonian.py:47-70.  Spatial methods (MP2, CID, CISD) give the same
energies as their spin-orbital forms and are run as those.  Used by the tests
to pin the oracle to the reference's golden energies and finite-difference
tensors.  The molecule/basis set-up is the product's host-side
``apyib_gb300.basis`` (pure Python, no device code).
"""
from __future__ import annotations

import numpy as np

from . import ints as OI
from . import port as OP


def ao_hamiltonian(geom, basis_name, F_el=(0.0, 0.0, 0.0), F_mag=(0.0, 0.0, 0.0)):
    """(S, T, V (complex, with field terms), ERI, E_nuc, nelec, basis) from the oracle integrals."""
    from apyib_gb300 import basis as B
    mol = B.parse_geometry(geom)
    bs = B.BasisSet.build(mol, basis_name)
    sh = OI.shells_of(bs)
    Tc = bs.cart_to_ao()

    def ao(M):
        return Tc @ M @ Tc.T
    S = ao(OI.one_electron(sh, "overlap"))
    T = ao(OI.one_electron(sh, "kinetic"))
    V = ao(OI.potential(sh, mol.Z.astype(float), mol.xyz)).astype(complex)
    G = np.einsum("pa,qb,rc,sd,abcd->pqrs", Tc, Tc, Tc, Tc, OI.eri(sh), optimize=True)
    if any(f != 0.0 for f in F_el):
        mu = OI.one_electron(sh, "dipole")
        for a in range(3):
            V = V - F_el[a] * ao(mu[a])
    if any(f != 0.0 for f in F_mag):
        L = OI.one_electron(sh, "angular momentum")
        for a in range(3):
            V = V - F_mag[a] * (-0.5j * ao(L[a]))
    E_nuc = mol.nuclear_repulsion_energy([-f for f in F_el])
    return S, T, V, G, E_nuc, int(mol.Z.sum()) - mol.charge, bs


def energy(parameters):
    """Total energy E_SCF + E_corr + E_nuc for parameters as the reference takes them."""
    S, T, V, G, E_nuc, nelec, bs = ao_hamiltonian(parameters["geom"], parameters["basis"],
                                                 parameters["F_el"], parameters["F_mag"])
    ndocc = nelec // 2
    E_scf, C, eps = OP.solve_scf(T, V, S, G, E_nuc, ndocc, parameters)
    E = E_scf + E_nuc
    method = parameters["method"].replace("_SO", "")
    if method == "RHF":
        return E
    nfzc = bs.n_frozen_core() if parameters.get("freeze_core") else 0
    C = C.astype(complex)
    F_MO, _ = OP.compute_F_MO(T + V, G, C, nfzc, ndocc, bs.nbf(), freeze_core=nfzc > 0)
    blk = OP.blocks_from_chemist(OP.compute_ERI_SO(OP.compute_ERI_MO(G, C[:, nfzc:])), 2 * (ndocc - nfzc))
    eo, ev = eps[nfzc:ndocc], eps[ndocc:]
    if method == "MP2":
        return E + OP.solve_mp2_so(blk, eo, ev)[0]
    return E + OP.solve_cisd_so(OP.compute_F_SO(F_MO), blk, eo, ev, parameters, singles=(method == "CISD"))[0]


def fd_hessian(parameters, h):
    """apyib/fin_diff.py:27-149 with the oracle energy (distinct geometries solved once)."""
    from apyib_gb300 import basis as B
    mol = B.parse_geometry(parameters["geom"])
    x0 = mol.geometry()
    n = 3 * mol.natom()
    cache = {}

    def E(moves):
        key = tuple(sorted((k, m) for k, m in moves.items() if m))
        if key not in cache:
            x = x0.copy()
            for k, m in key:
                x[k // 3, k % 3] += m * h
            mol.set_geometry(x)
            cache[key] = energy(dict(parameters, geom=mol.create_psi4_string_from_molecule()))
        return cache[key]
    g = {}
    for s in (1, -1):
        gs = np.zeros((n, n), dtype=complex)
        for a in range(n):
            for b in range(n):
                mp = {a: s}
                mp[b] = mp.get(b, 0) + 1
                mm = {a: s}
                mm[b] = mm.get(b, 0) - 1
                gs[a, b] = (E(mp) - E(mm)) / (2 * h)
        g[s] = gs
    return (g[1] - g[-1]) / (2 * h)


def fd_apt(parameters, h, f):
    """apyib/fin_diff.py:151-265 with the oracle energy."""
    from apyib_gb300 import basis as B
    mol = B.parse_geometry(parameters["geom"])
    x0 = mol.geometry()
    n = 3 * mol.natom()
    mu = {}
    for s in (1, -1):
        m = np.zeros((n, 3), dtype=complex)
        for a in range(n):
            x = x0.copy()
            x[a // 3, a % 3] += s * h
            mol.set_geometry(x)
            geom = mol.create_psi4_string_from_molecule()
            for b in range(3):
                e = []
                for sf in (1, -1):
                    F = [0.0, 0.0, 0.0]
                    F[b] = sf * f
                    e.append(energy(dict(parameters, geom=geom, F_el=F)))
                m[a, b] = -(e[0] - e[1]) / (2 * f)
        mu[s] = m
    return (mu[1] - mu[-1]) / (2 * h)
