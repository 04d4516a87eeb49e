"""The two water workloads of the benchmark definition from their geometry string,
through the public API (apyib_gb300.energy.energy: GPU integrals -> RHF -> MP2_SO /
CID_SO / CISD_SO), against the reference's own NumPy chain run on the same
(oracle) integrals (tests/golden/make_golden_configs.py -> configs_h2o.json):
H2O STO-3G zero field, and H2O cc-pVDZ with a 1e-4 a.u. magnetic field along z
(complex orbitals).  FP64: energies to 1e-10 Eh, amplitude norms to 1e-9
relative.  Mixed precision (3xTF32 tensor-core iterations + FP64-accurate
refinement): |dE| <= 1e-9 Eh against the same reference energies."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300.energy import energy  # noqa: E402

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "configs_h2o.json")))
CONV = dict(e_convergence=1e-12, d_convergence=1e-12, DIIS=True, max_iterations=120, freeze_core=False,
            F_el=[0.0, 0.0, 0.0])


def _run(g, method, precision=None):
    p = dict(CONV, geom=g["geom"], basis=g["basis"], F_mag=list(g["F_mag"]), method=method)
    if precision:
        p["precision"] = precision
    return energy(p)


@pytest.mark.parametrize("name", list(GOLD))
def test_fp64_chain_matches_reference(name):
    g = GOLD[name]
    for method, key, norms in (("MP2_SO", "E_mp2", {2: "mp2_t2_norm2"}), ("CID_SO", "E_cid", {2: "cid_t2_norm2"}),
                               ("CISD_SO", "E_cisd", {1: "cisd_t1_norm2", 2: "cisd_t2_norm2"})):
        E_list, T_list, C, basis = _run(g, method)
        assert abs(complex(E_list[0]) - complex(*g["E_scf"])) < 1e-10, (name, method, E_list[0])
        assert abs(complex(E_list[1]) - complex(*g[key])) < 1e-10, (name, method, E_list[1], g[key])
        assert abs(E_list[2] - g["E_nuc"]) < 1e-12
        for k, nk in norms.items():
            n2 = float(np.sum(np.abs(np.asarray(T_list[k])) ** 2))
            assert abs(n2 - g[nk]) <= 1e-9 * g[nk], (name, method, k, n2, g[nk])


@pytest.mark.parametrize("name", list(GOLD))
def test_mixed_precision_meets_energy_target(name):
    g = GOLD[name]
    for method, key in (("CID_SO", "E_cid"), ("CISD_SO", "E_cisd")):
        E_list, _, _, _ = _run(g, method, precision="mixed")
        assert abs(complex(E_list[1]) - complex(*g[key])) <= 1e-9, (name, method, E_list[1], g[key])
