"""AO integrals on the GPU and the whole path from a geometry string.

* agb_ao_one_electron / agb_ao_eri (+ the solid-harmonic transform) against the
  NumPy oracle (oracle/ints.py, itself pinned to the reference's
  apyib/integrals.py) for water in STO-3G (pure p), 6-31G(d) (Cartesian d) and
  cc-pVDZ (pure d), and an f shell;
* ``apyib_gb300.energy.energy(parameters)`` (Hamiltonian -> RHF -> MP2 / CID /
  CISD, spin-orbital and spatial) against every energy the reference's test
  suite asserts for these basis sets, to the reference's tolerance of 1e-11;
* a complex magnetic-field and an electric-field Hamiltonian against the
  oracle chain on the same inputs.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import basis as B  # noqa: E402
from apyib_gb300.energy import energy  # noqa: E402
from apyib_gb300.integrals import MintsHelper  # noqa: E402
from oracle import ints as OI  # noqa: E402
from oracle import port as OP  # noqa: E402
from tests.golden.reference_energies import CASES, GEOMS, H2O, PARAMS  # noqa: E402


def _oracle_ao(bs, kind):
    sh = OI.shells_of(bs)
    Tc = bs.cart_to_ao()
    if kind == "potential":
        return Tc @ OI.potential(sh, bs.molecule.Z.astype(float), bs.molecule.xyz) @ Tc.T
    if kind == "eri":
        return np.einsum("pa,qb,rc,sd,abcd->pqrs", Tc, Tc, Tc, Tc, OI.eri(sh), optimize=True)
    M = OI.one_electron(sh, kind)
    if M.ndim == 3:
        return np.stack([Tc @ m @ Tc.T for m in M])
    return Tc @ M @ Tc.T


@pytest.mark.parametrize("name", ["STO-3G", "6-31G(d)", "cc-pVDZ"])
def test_integrals_match_oracle(name):
    bs = B.BasisSet.build(B.parse_geometry(H2O), name)
    m = MintsHelper(bs)
    got = {"overlap": m.ao_overlap(), "kinetic": m.ao_kinetic(), "potential": m.ao_potential(),
           "dipole": np.stack(m.ao_dipole()), "nabla": np.stack(m.ao_nabla()),
           "angular momentum": np.stack(m.ao_angular_momentum()), "eri": m.ao_eri()}
    for kind, g in got.items():
        ref = _oracle_ao(bs, kind)
        assert g.shape == ref.shape, kind
        np.testing.assert_allclose(g, ref, atol=1e-12 * max(1.0, np.abs(ref).max()), rtol=0, err_msg=f"{name} {kind}")
    assert np.allclose(got["overlap"].np, got["overlap"])          # psi4 Matrix-style .np


def test_f_shell_and_origin():
    """An f shell (l = 3, the largest supported) and a shifted operator origin."""
    B.register_basis("test-spdf", """
****
H     0
S   2   1.00
      1.3000000              0.4000000
      0.3000000              0.7000000
P   1   1.00
      0.9000000              1.0000000
****
O     0
F   1   1.00
      0.8000000              1.0000000
****
""", pure=True)
    mol = B.parse_geometry("O 0.1 -0.2 0.05\nH 1.4 0.9 -0.3\nunits bohr\n")
    bs = B.BasisSet.build(mol, "test-spdf")
    m = MintsHelper(bs)
    origin = (0.3, -0.1, 0.2)
    sh = OI.shells_of(bs)
    Tc = bs.cart_to_ao()
    for kind, got in (("overlap", m.ao_overlap()), ("kinetic", m.ao_kinetic()), ("potential", m.ao_potential())):
        ref = _oracle_ao(bs, kind)
        np.testing.assert_allclose(got, ref, atol=1e-12 * max(1.0, np.abs(ref).max()), rtol=0, err_msg=kind)
    # dipole about a shifted origin: -<r - O> = -<r> + O S
    S = Tc @ OI.one_electron(sh, "overlap") @ Tc.T
    dip0 = np.stack([Tc @ x @ Tc.T for x in OI.one_electron(sh, "dipole")])
    dipO = np.stack(m.ao_dipole(origin=origin))
    np.testing.assert_allclose(dipO, dip0 + np.asarray(origin)[:, None, None] * S[None], atol=1e-12, rtol=0)
    eri = m.ao_eri()
    ref = _oracle_ao(bs, "eri")
    np.testing.assert_allclose(eri, ref, atol=1e-12 * np.abs(ref).max(), rtol=0)


def _method_variants():
    out = []
    for c in CASES:
        if c[2] == "RHF":
            out.append((c, "RHF"))
        else:
            out.append((c, c[2] + "_SO"))
            out.append((c, c[2]))
    return out


VARIANTS = _method_variants()


@pytest.mark.parametrize("case,method", VARIANTS, ids=[f"{c[0]}-{m}" for c, m in VARIANTS])
def test_energy_driver_reproduces_reference_golden(case, method):
    cid, where, _, basis, mol_key, fc, golden = case
    params = dict(PARAMS, geom=GEOMS[mol_key], basis=basis, method=method, freeze_core=fc)
    E_list, T_list, C, bs = energy(params)
    E = complex(E_list[0]).real + complex(E_list[1]).real + E_list[2]
    assert abs(E - golden) < 1e-11, (cid, method, where, E, golden, E - golden)


@pytest.mark.parametrize("field", ["magnetic", "electric"])
def test_field_hamiltonian_matches_oracle_chain(field):
    """Complex (magnetic) and real (electric) field terms of apyib/hamiltonian.py:47-70
    through SCF and CISD_SO against the oracle chain on the same inputs."""
    from apyib_gb300.hamiltonian import Hamiltonian
    F = [0.0, 0.0, 0.0]
    F[1] = 0.002
    params = dict(PARAMS, geom=H2O, basis="STO-3G", method="CISD_SO", freeze_core=False,
                  F_mag=F if field == "magnetic" else [0.0] * 3, F_el=F if field == "electric" else [0.0] * 3)
    H = Hamiltonian(params)
    E_list, _, _, _ = energy(params)
    bs = B.BasisSet.build(B.parse_geometry(H2O), "STO-3G")
    sh = OI.shells_of(bs)
    Tc = bs.cart_to_ao()
    S = Tc @ OI.one_electron(sh, "overlap") @ Tc.T
    T = Tc @ OI.one_electron(sh, "kinetic") @ Tc.T
    V = (Tc @ OI.potential(sh, bs.molecule.Z.astype(float), bs.molecule.xyz) @ Tc.T).astype(complex)
    G = np.einsum("pa,qb,rc,sd,abcd->pqrs", Tc, Tc, Tc, Tc, OI.eri(sh), optimize=True)
    if field == "magnetic":
        L = np.stack([Tc @ x @ Tc.T for x in OI.one_electron(sh, "angular momentum")])
        V = V - F[1] * (-0.5j * L[1])
        E_nuc = bs.molecule.nuclear_repulsion_energy()
    else:
        mu = np.stack([Tc @ x @ Tc.T for x in OI.one_electron(sh, "dipole")])
        V = V - F[1] * mu[1]
        E_nuc = bs.molecule.nuclear_repulsion_energy([-f for f in F])
    np.testing.assert_allclose(H.V, V, atol=1e-12, rtol=0)
    assert abs(H.E_nuc - E_nuc) < 1e-12
    ndocc = 5
    E_scf, C, eps = OP.solve_scf(T, V, S, G, E_nuc, ndocc, PARAMS)
    F_MO, _ = OP.compute_F_MO(T + V, G, C, 0, ndocc, bs.nbf())
    blk = OP.blocks_from_chemist(OP.compute_ERI_SO(OP.compute_ERI_MO(G, C)), 2 * ndocc)
    Ec = OP.solve_cisd_so(OP.compute_F_SO(F_MO), blk, eps[:ndocc], eps[ndocc:], PARAMS)[0]
    assert abs(E_list[0] - E_scf) < 1e-10
    assert abs(E_list[1] - Ec) < 1e-10
