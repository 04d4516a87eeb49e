"""Finite-difference drivers on the GPU energy path (apyib_gb300.fin_diff), from
geometry strings, against the reference's own golden tensors:
every Hessian of apyib/tests/test_009_Hessian.py (RHF, MP2, MP2_SO, CID, CID_SO at
STO-3G; CISD and CISD_SO at 6-31G, the last one skipped by the reference as too
slow) and every atomic polar tensor of apyib/tests/test_010_APT.py, to the
reference's tolerances; and the nuclear-gradient, magnetic-field-gradient and
AAT-input drivers (phase-corrected wavefunctions)."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import basis as B  # noqa: E402
from apyib_gb300.energy import energy  # noqa: E402
from apyib_gb300.fin_diff import finite_difference  # noqa: E402
from apyib_gb300.utils import compute_mo_overlap  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fd_goldens.json")))
CASES = [(k, c) for k in ("hessian", "apt") for c in GOLD[k]]


def _params(case):
    p = dict(case["parameters"])
    p["geom"] = GOLD["molecules"][p["geom"]["moldict"]]
    p["F_el"] = list(p["F_el"])
    p["F_mag"] = list(p["F_mag"])
    return p


@pytest.mark.parametrize("kind,case", CASES, ids=[c["name"] for _, c in CASES])
def test_fd_tensor_matches_reference_golden(kind, case):
    p = _params(case)
    E_list, T_list, C, basis = energy(p)
    fd = finite_difference(p, basis, C)
    ref = np.array(case["ref"])
    if kind == "hessian":
        n = int(round(np.sqrt(ref.size)))
        got = fd.compute_Hessian(*case["steps"])
        ref = ref.reshape(n, n)
    else:
        got = fd.compute_APT(*case["steps"])
    assert np.abs(got - ref).max() < case["tol"], (case["name"], np.abs(got - ref).max())


@pytest.mark.parametrize("method,mol", [("RHF", "H2O_C4_HF"), ("MP2_SO", "H2O_C4_MP2"), ("CID_SO", "H2O_C4_CID")])
def test_gradients_and_aat_inputs(method, mol):
    """At the geometry CFOUR optimised for the same method and basis the FD nuclear
    gradient vanishes; a closed-shell ground state has no magnetic moment, so the
    field gradient vanishes too; the AAT inputs are phase-aligned wavefunctions."""
    p = dict(GOLD["hessian"][0]["parameters"], geom=GOLD["molecules"][mol], method=method,
             F_el=[0.0, 0.0, 0.0], F_mag=[0.0, 0.0, 0.0])
    E_list, T_list, C, basis = energy(p)
    fd = finite_difference(p, basis, C)
    g, pos_C, neg_C, pos_b, neg_b, pos_T, neg_T = fd.compute_Nuclear_Gradient(1e-3)
    assert g.shape == (3, 3) and np.abs(g).max() < 2e-5, g
    assert np.abs(g.sum(axis=0)).max() < 1e-7                 # translational invariance
    gm, mpos_C, mneg_C, _, _, _, _ = fd.compute_Magnetic_Field_Gradient(1e-4)
    assert np.abs(gm).max() < 1e-7, gm
    ndocc = 5
    for Cx, bx in ((pos_C[4], pos_b[4]), (mpos_C[1], basis)):
        S = compute_mo_overlap(ndocc, basis.nbf(), basis, C, bx, Cx)
        d = np.diagonal(S)[:ndocc]
        assert np.all(np.abs(d.imag) < 1e-12) and np.all(d.real > 0.9)
    out = fd.compute_AAT(1e-4, 1e-4)
    assert len(out) == 12 and len(out[0]) == 9 and len(out[6]) == 3
