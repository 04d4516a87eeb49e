"""CPU checks of the AO integral oracle and the basis/molecule host logic.

* one-electron integrals of the oracle against the reference's own
  apyib/integrals.py run on the same shells (tests/golden/oei_h2o_631gd.npz);
* the whole CPU oracle chain (oracle integrals -> oracle SCF -> MP2_SO / CID_SO /
  CISD_SO of oracle/port.py) against every energy the reference's test suite
  asserts at STO-3G, 6-31G, 6-31G(d) and cc-pVDZ (tests/golden/reference_energies.py),
  to the reference's own tolerance of 1e-11 hartree;
* molecule parsing, nuclear repulsion, normalisation and the solid-harmonic transform.
"""
import functools
import os

import numpy as np
import pytest

from apyib_gb300 import basis as B
from oracle import ints as OI
from oracle import port as OP
from tests.golden.reference_energies import CASES, GEOMS, H2O, PARAMS

HERE = os.path.dirname(os.path.abspath(__file__))


def test_one_electron_matches_reference_integrals_py():
    g = np.load(os.path.join(HERE, "golden", "oei_h2o_631gd.npz"))
    bs = B.BasisSet.build(B.parse_geometry(H2O), "6-31G(d)", puream=False)
    np.testing.assert_array_equal(np.concatenate([sh.exps for sh in bs.shells]), g["exps"])
    np.testing.assert_allclose(np.concatenate([sh.coefs for sh in bs.shells]), g["coefs"], rtol=1e-15, atol=0)
    sh = OI.shells_of(bs)
    for kind in ("overlap", "kinetic", "dipole", "nabla", "angular_momentum"):
        M = OI.one_electron(sh, kind.replace("_", " "))
        np.testing.assert_allclose(M, g[kind], atol=1e-13, rtol=0, err_msg=kind)


def test_molecule_and_nuclear_repulsion():
    mol = B.parse_geometry(H2O)
    assert mol.symbols == ["O", "H", "H"] and list(mol.Z) == [8, 1, 1]
    e0 = mol.nuclear_repulsion_energy()
    R = mol.xyz
    pair = (8 / np.linalg.norm(R[0] - R[1]) + 8 / np.linalg.norm(R[0] - R[2]) + 1 / np.linalg.norm(R[1] - R[2]))
    assert abs(e0 - pair) < 1e-14 and abs(e0 - 8.0023670618) < 1e-9
    # a field adds field . sum_A Z_A R_A
    f = np.array([0.01, -0.02, 0.03])
    assert abs(mol.nuclear_repulsion_energy(f) - e0 - f @ (mol.Z[:, None] * mol.xyz).sum(0)) < 1e-14
    ang = B.parse_geometry("H 0 0 0\nH 0 0 0.74\n")          # psi4's default units: angstrom
    assert abs(ang.xyz[1, 2] - 0.74 / 0.52917721067) < 1e-12
    assert B.parse_geometry("0 1\nO 0 0 0\nunits bohr\n").natom() == 1
    with pytest.raises(ValueError):
        B.parse_geometry("Xx 0 0 0\n")


def test_basis_counts_and_frozen_core():
    mol = B.parse_geometry(H2O)
    for name, nbf, ncart in (("STO-3G", 7, 7), ("6-31G", 13, 13), ("6-31G(d)", 19, 19), ("cc-pVDZ", 24, 25)):
        bs = B.BasisSet.build(mol, name)
        assert (bs.nbf(), bs.ncart()) == (nbf, ncart), name
    assert B.BasisSet.build(mol, "cc-pVDZ", freeze_core=True).n_frozen_core() == 1
    assert B.BasisSet.build(mol, "cc-pVDZ").n_frozen_core() == 0
    with pytest.raises(KeyError):
        B.BasisSet.build(mol, "no-such-basis")


@pytest.mark.parametrize("l", [1, 2, 3])
def test_normalisation_and_pure_transform(l):
    exps, coefs = np.array([3.0, 0.7, 0.2]), np.array([0.2, 0.5, 0.4])
    sh = [(l, np.zeros(3), exps, B.normalized_coefficients(l, exps, coefs))]
    S = OI.one_electron(sh, "overlap")
    comps = B.cartesian_components(l)
    for k, c in enumerate(comps):
        if max(c) == l:
            assert abs(S[k, k] - 1.0) < 1e-14
    T = B.pure_transform(l)
    np.testing.assert_allclose(T @ S @ T.T, np.eye(2 * l + 1), atol=1e-14)


@functools.lru_cache(maxsize=None)
def _ao(mol_key, basis):
    mol = B.parse_geometry(GEOMS[mol_key])
    bs = B.BasisSet.build(mol, basis)
    sh = OI.shells_of(bs)
    Tc = bs.cart_to_ao()
    S = Tc @ OI.one_electron(sh, "overlap") @ Tc.T
    T = Tc @ OI.one_electron(sh, "kinetic") @ Tc.T
    V = Tc @ OI.potential(sh, mol.Z.astype(float), mol.xyz) @ Tc.T
    G = np.einsum("pa,qb,rc,sd,abcd->pqrs", Tc, Tc, Tc, Tc, OI.eri(sh), optimize=True)
    return mol, bs, S, T, V, G


@functools.lru_cache(maxsize=None)
def _scf(mol_key, basis):
    mol, bs, S, T, V, G = _ao(mol_key, basis)
    E_nuc = mol.nuclear_repulsion_energy()
    ndocc = int(mol.Z.sum()) // 2
    E, C, eps = OP.solve_scf(T, V.astype(complex), S, G, E_nuc, ndocc, PARAMS)
    return E.real, E_nuc, C.astype(complex), eps, ndocc


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_reproduces_reference_golden_energy(case):
    cid, where, method, basis, mol_key, fc, golden = case
    mol, bs, S, T, V, G = _ao(mol_key, basis)
    E_scf, E_nuc, C, eps, ndocc = _scf(mol_key, basis)
    E = E_scf + E_nuc
    if method != "RHF":
        nfzc = 1 if fc else 0
        nbf = bs.nbf()
        F_MO, _ = OP.compute_F_MO((T + V).astype(complex), G, C, nfzc, ndocc, nbf, freeze_core=fc)
        blk = OP.blocks_from_chemist(OP.compute_ERI_SO(OP.compute_ERI_MO(G, C[:, nfzc:])), 2 * (ndocc - nfzc))
        eo, ev = eps[nfzc:ndocc], eps[ndocc:]
        if method == "MP2":
            Ec, _ = OP.solve_mp2_so(blk, eo, ev)
        else:
            Ec = OP.solve_cisd_so(OP.compute_F_SO(F_MO), blk, eo, ev, PARAMS, singles=(method == "CISD"))[0]
        E += Ec.real
    assert abs(E - golden) < 1e-11, (cid, where, E, golden, E - golden)
