"""Analytic nuclear gradients (apyib_gb300.gradient: one SCF + one CI solve, the
Hellmann-Feynman densities, derivative integrals and the CPHF orbital response)
against central finite differences of complete GPU calculations
(fin_diff.compute_Nuclear_Gradient at 1e-3 and 5e-4 bohr, Richardson-combined),
for RHF, MP2 (through its Lagrangian densities), CID and CISD (spin-orbital and
spatial) of water away from its equilibrium geometry, to 1e-6 relative; atomic polar
tensors from them against the reference's finite-difference goldens."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300.energy import energy  # noqa: E402
from apyib_gb300.fin_diff import finite_difference  # noqa: E402
from apyib_gb300.gradient import nuclear_gradient  # noqa: E402
from tests.golden.reference_energies import H2O, PARAMS  # noqa: E402

CASES = [("STO-3G", "RHF"), ("STO-3G", "CISD_SO"), ("STO-3G", "CID"), ("6-31G", "CISD"), ("cc-pVDZ", "RHF"),
         ("cc-pVDZ", "CID_SO"), ("STO-3G", "MP2_SO"), ("6-31G", "MP2")]


@pytest.mark.parametrize("basis,method", CASES, ids=[f"{b}-{m}" for b, m in CASES])
def test_analytic_gradient_matches_finite_differences(basis, method):
    p = dict(PARAMS, geom=H2O, basis=basis, method=method, freeze_core=False)
    g, parts = nuclear_gradient(p, return_parts=True)
    E_list, _, C, bs = energy(p)
    E = complex(E_list[0]) + complex(E_list[1]) + E_list[2]
    assert abs(parts["E"] - E) < 1e-10
    fd = finite_difference(p, bs, C)
    g1 = fd.compute_Nuclear_Gradient(1e-3)[0]
    g2 = fd.compute_Nuclear_Gradient(5e-4)[0]
    gfd = (4 * g2 - g1) / 3
    err = np.abs(g - gfd).max()
    assert err <= 1e-6 * np.abs(gfd).max() + 1e-9, (basis, method, err, g, gfd)
    assert np.abs(g.sum(axis=0)).max() < 1e-9                      # translational invariance


def _apt_cases():
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fd_goldens.json")))
    cases = [c for c in gold["apt"] if c["parameters"]["method"] in ("RHF", "MP2", "MP2_SO", "CID", "CID_SO")]
    return gold, cases


APT_GOLD, APT_CASES = _apt_cases()


@pytest.mark.parametrize("case", APT_CASES, ids=[c["name"] for c in APT_CASES])
def test_semianalytic_apt_matches_reference_golden(case):
    """APTs from analytic gradients in +-field (Richardson, 5e-4 and 1e-3 a.u.) against the reference's
    finite-difference golden (apyib/tests/test_010_APT.py) to its tolerance."""
    from apyib_gb300.gradient import apt
    p = dict(case["parameters"])
    p["geom"] = APT_GOLD["molecules"][p["geom"]["moldict"]]
    P = apt(p)
    err = np.abs(P - np.array(case["ref"])).max()
    assert err < case["tol"], (case["name"], err)


def test_gradient_in_electric_field():
    p = dict(PARAMS, geom=H2O, basis="STO-3G", method="CISD_SO", freeze_core=False, F_el=[0.0, 0.003, -0.002])
    g = nuclear_gradient(p)
    E_list, _, C, bs = energy(p)
    fd = finite_difference(p, bs, C)
    g1, g2 = fd.compute_Nuclear_Gradient(1e-3)[0], fd.compute_Nuclear_Gradient(5e-4)[0]
    gfd = (4 * g2 - g1) / 3
    assert np.abs(g - gfd).max() <= 1e-6 * np.abs(gfd).max() + 1e-9


@pytest.mark.parametrize("case", APT_GOLD["apt_analytic"], ids=[c["name"] for c in APT_GOLD["apt_analytic"]])
def test_apt_matches_reference_analytic_golden(case):
    """RHF APTs of NH3 / 6-31G* (apyib/tests/test_022_RHF_Analytic_APT.py): length gauge from
    analytic gradients in +-field (Richardson over two field steps), velocity gauge from the
    velocity-operator CPHF response and the determinant overlap derivative; to the reference's 1e-6."""
    from apyib_gb300.analytic_apts import analytic_derivative
    ad = analytic_derivative(dict(case["parameters"]))
    P = ad.compute_RHF_APTs_VG() if case["name"].endswith("_VG") else ad.compute_RHF_APTs_LG()
    err = np.abs(P - np.array(case["ref"])).max()
    assert err < case["tol"], (case["name"], err)
