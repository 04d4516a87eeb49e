"""Nuclear first derivatives of the AO integrals (agb_ao_one_electron_deriv,
agb_ao_eri_deriv) against Richardson central differences (steps 2e-3 and 1e-3
bohr) of the GPU integrals at displaced geometries (those integrals are pinned to
the oracle in test_gpu_ints.py), for water in STO-3G, 6-31G(d) (Cartesian d) and
cc-pVDZ (pure d); translational invariance (the derivatives over all atoms sum to
zero); and the half-derivative overlaps (LEFT + RIGHT = the full derivative)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402
from apyib_gb300 import basis as B  # noqa: E402
from apyib_gb300.integrals import MintsHelper  # noqa: E402
from tests.golden.reference_energies import H2O  # noqa: E402

KINDS = {"OVERLAP": _lib.OEI_OVERLAP, "KINETIC": _lib.OEI_KINETIC, "POTENTIAL": _lib.OEI_POTENTIAL}


def _ints_at(mol0, name, k, c, d):
    mol = B.parse_geometry(mol0.create_psi4_string_from_molecule())
    x = mol.geometry()
    x[k, c] += d
    mol.set_geometry(x)
    m = MintsHelper(B.BasisSet.build(mol, name))
    return {"OVERLAP": m.ao_overlap(), "KINETIC": m.ao_kinetic(), "POTENTIAL": m.ao_potential(), "ERI": m.ao_eri(),
            "DIPOLE": np.stack(m.ao_dipole())}


@pytest.mark.parametrize("name", ["STO-3G", "6-31G(d)", "cc-pVDZ"])
def test_derivatives_match_central_differences(name):
    mol = B.parse_geometry(H2O)
    m = MintsHelper(B.BasisSet.build(mol, name))
    got = {kk: m.oei_deriv_all(v).cpu().numpy() for kk, v in KINDS.items()}
    got["ERI"] = m.eri_deriv_all().cpu().numpy()
    dip = m.oei_deriv_all(_lib.OEI_DIPOLE).cpu().numpy()                # [atom, c, beta, n, n]
    S = m.ao_overlap()
    for c in range(3):                                   # rigid translation: d(-<r>)/dR summed = -S
        for beta in range(3):
            np.testing.assert_allclose(dip[:, c, beta].sum(axis=0), -S * (c == beta), atol=1e-11, rtol=0)
    got["DIPOLE"] = dip
    for kk, g in got.items():
        if kk == "DIPOLE":
            continue
        tot = g.sum(axis=0)                                       # translational invariance
        assert np.abs(tot).max() < 1e-11 * max(1.0, np.abs(g).max()), (name, kk, np.abs(tot).max())
    h = 2e-3
    for k, c in ((0, 1), (1, 0), (2, 2)):
        ints = {d: _ints_at(mol, name, k, c, d) for d in (h, -h, h / 2, -h / 2)}
        for kk, g in got.items():
            d1 = (ints[h][kk] - ints[-h][kk]) / (2 * h)
            d2 = (ints[h / 2][kk] - ints[-h / 2][kk]) / h
            fd = (4 * d2 - d1) / 3
            err = np.abs(g[k, c] - fd).max()
            assert err < 1e-9 * max(1.0, np.abs(fd).max()), (name, kk, k, c, err)


def test_half_derivative_overlap():
    mol = B.parse_geometry(H2O)
    m = MintsHelper(B.BasisSet.build(mol, "cc-pVDZ"))
    full = m.oei_deriv_all(_lib.OEI_OVERLAP)
    for atom in range(3):
        L = np.stack(m.ao_overlap_half_deriv1("LEFT", atom))
        R = np.stack(m.ao_overlap_half_deriv1("RIGHT", atom))
        np.testing.assert_allclose(L + R, full[atom].cpu().numpy(), atol=1e-13, rtol=0)
        np.testing.assert_allclose(R, np.swapaxes(L, 1, 2), atol=0, rtol=0)
    d = m.ao_oei_deriv1("kinetic", 1)
    assert len(d) == 3 and d[0].shape == (24, 24)
