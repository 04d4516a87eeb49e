"""The oracle chain (oracle/chain.py: oracle integrals -> SCF -> CID_SO) run through
the reference's finite-difference recipes against the reference's own golden
Hessians (apyib/tests/test_009_Hessian.py) and atomic polar tensors
(apyib/tests/test_010_APT.py), extracted by tests/golden/make_golden_fd.py, to
the reference's tolerances (1e-6 and 1e-5)."""
import json
import os

import numpy as np
import pytest

from oracle import chain

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fd_goldens.json")))
PICK = [(k, c) for k in ("hessian", "apt") for c in GOLD[k]
        if not c["skip"] and c["parameters"]["method"] in ("RHF", "CID_SO")]


@pytest.mark.parametrize("kind,case", PICK, ids=[c["name"] for _, c in PICK])
def test_oracle_fd_tensor_matches_reference_golden(kind, case):
    p = dict(case["parameters"])
    p["geom"] = GOLD["molecules"][p["geom"]["moldict"]]
    ref = np.array(case["ref"])
    if kind == "hessian":
        n = int(round(np.sqrt(ref.size)))
        got = chain.fd_hessian(p, *case["steps"])
        ref = ref.reshape(n, n)
    else:
        got = chain.fd_apt(p, *case["steps"])
    assert np.abs(got - ref).max() < case["tol"], (case["name"], np.abs(got - ref).max())
