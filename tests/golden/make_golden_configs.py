"""Reference energies for the two water workloads the benchmark is defined on.

* H2O STO-3G (O 0,0,0.1173; H 0,+-0.7572,-0.4692 angstrom), zero field;
* H2O cc-pVDZ, same geometry, magnetic field 1e-4 a.u. along z in the core
  Hamiltonian (the imaginary i B.L / 2 term of apyib/hamiltonian.py:55-70).

The AO integrals come from the oracle (oracle/chain.py, pinned to the
reference's golden energies); the unmodified reference modules
(apyib/hf_wfn.py, mp2_wfn.py, ci_wfn.py, utils.py, loaded by ref_loader with a
stub psi4) run RHF -> MP2_SO -> CID_SO -> CISD_SO on them through a duck-typed
Hamiltonian.  Stored: energies and the phase-invariant amplitude norms
sum |t1|^2, sum |t2|^2 (the orbitals are complex, so amplitudes themselves
depend on the arbitrary MO phases).  Output: tests/golden/configs_h2o.json.

    APYIB_REF=/path/to/apyib-checkout python tests/golden/make_golden_configs.py
"""
import contextlib
import io
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle import chain  # noqa: E402
from ref_loader import load_reference  # noqa: E402

GEOM = """
O 0.0  0.0     0.1173
H 0.0  0.7572 -0.4692
H 0.0 -0.7572 -0.4692
units angstrom
no_com
no_reorient
symmetry c1
"""
CONFIGS = {
    "h2o_sto3g": dict(basis="STO-3G", F_mag=[0.0, 0.0, 0.0]),
    "h2o_ccpvdz_bz": dict(basis="cc-pVDZ", F_mag=[0.0, 0.0, 1e-4]),
}
CONV = dict(e_convergence=1e-12, d_convergence=1e-12, DIIS=True, max_iterations=120, freeze_core=False,
            F_el=[0.0, 0.0, 0.0])


def run(name, cfg, ref):
    S, T, V, G, E_nuc, nelec, bs = chain.ao_hamiltonian(GEOM, cfg["basis"], [0.0, 0.0, 0.0], cfg["F_mag"])
    nbf = bs.nbf()
    basis = types.SimpleNamespace(nbf=lambda: nbf, n_frozen_core=lambda: 0)
    mol = types.SimpleNamespace(natom=lambda: 1, true_atomic_number=lambda a: nelec)
    H = types.SimpleNamespace(basis_set=basis, molecule=mol, E_nuc=E_nuc, S=S, T=T, V=V, ERI=G)
    p = dict(CONV, geom=GEOM, basis=cfg["basis"], F_mag=cfg["F_mag"])
    out = {"geom": GEOM, "basis": cfg["basis"], "F_mag": cfg["F_mag"], "nbf": nbf, "E_nuc": E_nuc}
    with contextlib.redirect_stdout(io.StringIO()):
        wfn = ref.hf_wfn.hf_wfn(H)
        E_scf, C = wfn.solve_SCF(dict(p, method="RHF"))
        E_mp2, t2 = ref.mp2_wfn.mp2_wfn(dict(p, method="MP2_SO"), wfn).solve_MP2_SO()
        out["mp2_t2_norm2"] = float(np.sum(np.abs(t2) ** 2))
        E_cid, t2 = ref.ci_wfn.ci_wfn(dict(p, method="CID_SO"), wfn).solve_CID_SO()
        out["cid_t2_norm2"] = float(np.sum(np.abs(t2) ** 2))
        E_cisd, t1, t2 = ref.ci_wfn.ci_wfn(dict(p, method="CISD_SO"), wfn).solve_CISD_SO()
        out["cisd_t1_norm2"] = float(np.sum(np.abs(t1) ** 2))
        out["cisd_t2_norm2"] = float(np.sum(np.abs(t2) ** 2))
    for k, v in (("E_scf", E_scf), ("E_mp2", E_mp2), ("E_cid", E_cid), ("E_cisd", E_cisd)):
        out[k] = [float(np.real(v)), float(np.imag(v))]
    print(name, {k: v for k, v in out.items() if k.startswith("E_")}, flush=True)
    return out


def main():
    ref = load_reference()
    data = {name: run(name, cfg, ref) for name, cfg in CONFIGS.items()}
    with open(os.path.join(HERE, "configs_h2o.json"), "w") as f:
        json.dump(data, f, indent=1)


if __name__ == "__main__":
    main()
