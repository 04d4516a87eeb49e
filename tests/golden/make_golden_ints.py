"""Generate tests/golden/oei_h2o_631gd.npz with the reference's own one-electron
integral code.

apyib/integrals.py:9-146 (``one_electron_integral``) computes overlap, dipole,
nabla, angular-momentum and kinetic integrals over Cartesian Gaussians from
psi4's shell objects.  This script loads that file with a stub ``psi4`` whose
``geometry`` / ``BasisSet.build`` return the molecule and shells of
``apyib_gb300.basis`` (6-31G(d) water: s, p and Cartesian d shells) and stores
the reference's matrices.  ``tests/test_oracle_ints.py`` checks the NumPy
oracle against them, and the GPU tests check the CUDA kernels against the
oracle.

Run where the reference sources are available:
    APYIB_REF=/path/to/apyib-checkout python tests/golden/make_golden_ints.py
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from apyib_gb300 import basis as B  # noqa: E402
from tests.golden.reference_energies import H2O  # noqa: E402

REF_ROOT = os.environ.get("APYIB_REF")
if not REF_ROOT:
    raise SystemExit("set APYIB_REF to an apyib source checkout (the directory holding apyib/)")
BASIS = "6-31G(d)"
KINDS = ("overlap", "kinetic", "dipole", "nabla", "angular momentum")


class _Mat:
    def __init__(self, a):
        self.np = np.asarray(a)


class _Mol:
    def __init__(self, mol):
        self.m = mol

    def natom(self):
        return self.m.natom()

    def geometry(self):
        return _Mat(self.m.xyz)

    def center_of_mass(self):
        return [0.0, 0.0, 0.0]


class _Shell:
    def __init__(self, sh):
        self.function_index = sh.cart0
        self.am = sh.l
        self.nprimitive = sh.nprimitive
        self.ncartesian = sh.ncart
        self.ncenter = sh.atom
        self._sh = sh

    def coef(self, k):
        return float(self._sh.coefs[k])

    def exp(self, k):
        return float(self._sh.exps[k])


class _Basis:
    def __init__(self, bs):
        self.bs = bs

    def nshell(self):
        return self.bs.nshell()

    def nao(self):
        return self.bs.ncart()

    def shell(self, k):
        return _Shell(self.bs.shells[k])


def load_reference_integrals(bs_of_geom):
    psi4 = types.ModuleType("psi4")
    psi4.geometry = lambda text: _Mol(B.parse_geometry(text))
    psi4.set_options = lambda opts: None
    psi4.core = types.SimpleNamespace(BasisSet=types.SimpleNamespace(
        build=lambda mol, quiet=True: _Basis(bs_of_geom(mol.m))))
    sys.modules["psi4"] = psi4
    path = os.path.join(REF_ROOT, "apyib", "integrals.py")
    spec = importlib.util.spec_from_file_location("apyib_ref_integrals", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    build = lambda mol: B.BasisSet.build(mol, BASIS, puream=False)  # noqa: E731
    ref = load_reference_integrals(build)
    params = {"geom": H2O, "basis": BASIS}
    out = {}
    for kind in KINDS:
        out[kind.replace(" ", "_")] = ref.one_electron_integral(params, kind, spherical_transform=False)
    bs = build(B.parse_geometry(H2O))
    out["exps"] = np.concatenate([sh.exps for sh in bs.shells])
    out["coefs"] = np.concatenate([sh.coefs for sh in bs.shells])
    path = os.path.join(HERE, "oei_h2o_631gd.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
