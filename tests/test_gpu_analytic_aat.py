"""Analytic atomic axial tensors (apyib_gb300.analytic_aats: CPHF orbital responses,
amplitude responses, overlap terms as contractions) against the golden AATs of
apyib/tests/test_018_RHF_Analytic_AAT.py, test_019_MP2_Analytic_AAT.py,
test_020_CID_Analytic_AAT.py and test_021_CISD_Analytic_AAT.py (H2O2 STO-3G, H2O 6-31G*;
all-electron and frozen core; the canonical and non-canonical goldens are equal), extracted
by tests/golden/make_golden_analytic_aat.py, to the reference's tolerance 1e-6."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300.analytic_aats import analytic_derivative  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                   "analytic_aat_goldens.json")))
CASES = [c for c in GOLD["cases"] if c["kwargs"].get("orbitals") == "canonical"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_analytic_aat_matches_reference_golden(case):
    p = dict(case["parameters"])
    g = p["geom"]
    p["geom"] = g["text"] if "text" in g else GOLD["molecules"][g["moldict"]]
    ad = analytic_derivative(p)
    aat = getattr(ad, case["call"])(**case["kwargs"])
    ref = np.array(case["ref"])
    err = np.abs(aat - ref).max()
    assert err < case["tol"], (case["name"], err, aat, ref)


MIXED = [c for c in CASES if c["parameters"]["method"] in ("CID", "CISD")]


@pytest.mark.parametrize("case", MIXED, ids=[c["name"] for c in MIXED])
def test_analytic_aat_mixed_precision_matches_golden(case):
    """precision='mixed' (mixed amplitude solve, FP64-accurate tensor-core / double-float
    residuals for the responses) reproduces the same goldens to the same tolerance."""
    p = dict(case["parameters"])
    g = p["geom"]
    p["geom"] = g["text"] if "text" in g else GOLD["molecules"][g["moldict"]]
    ad = analytic_derivative(p)
    aat = getattr(ad, case["call"])(precision="mixed", **case["kwargs"])
    err = np.abs(aat - np.array(case["ref"])).max()
    assert err < case["tol"], (case["name"], err)
