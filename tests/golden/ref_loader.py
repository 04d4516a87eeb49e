"""Load the reference apyib hot-path modules (utils, hamiltonian, hf_wfn,
mp2_wfn, ci_wfn) from a source checkout with a stub ``psi4`` module.

This is fixture-generation infrastructure only: it runs where the reference
sources are available (the ``APYIB_REF`` environment variable names the
checkout; there is no default) and is never imported by the GPU tests, ``smoke()`` or
``bench.py``.  The reference imports ``psi4`` at module level
(apyib/utils.py:4, apyib/hf_wfn.py:3, apyib/mp2_wfn.py:3, apyib/ci_wfn.py:3,
apyib/hamiltonian.py:3) but the hot-path functions never call it once a
duck-typed Hamiltonian is supplied (apyib/utils.py:186, apyib/hf_wfn.py:20,30).
"""
import importlib.util
import os
import sys
import types



def reference_root():
    """The apyib source checkout named by ``APYIB_REF`` (required)."""
    root = os.environ.get("APYIB_REF")
    if not root:
        raise SystemExit("set APYIB_REF to an apyib source checkout (the directory holding apyib/)")
    return root


REF_ROOT = reference_root()


def _stub_psi4():
    if "psi4" in sys.modules:
        return
    psi4 = types.ModuleType("psi4")
    psi4.core = types.SimpleNamespace()
    sys.modules["psi4"] = psi4


def load_reference():
    """Return a namespace with the reference modules, loaded by file path."""
    _stub_psi4()
    pkg_dir = os.path.join(REF_ROOT, "apyib")
    if not os.path.isdir(pkg_dir):
        raise FileNotFoundError(f"reference sources not found at {pkg_dir}")
    if "apyib" not in sys.modules or not hasattr(sys.modules["apyib"], "_ref_loaded"):
        pkg = types.ModuleType("apyib")
        pkg.__path__ = [pkg_dir]
        pkg._ref_loaded = True
        sys.modules["apyib"] = pkg
    mods = {}
    for name in ("utils", "hamiltonian", "hf_wfn", "mp2_wfn", "ci_wfn"):
        full = f"apyib.{name}"
        if full not in sys.modules:
            spec = importlib.util.spec_from_file_location(full, os.path.join(pkg_dir, f"{name}.py"))
            mod = importlib.util.module_from_spec(spec)
            sys.modules[full] = mod
            spec.loader.exec_module(mod)
            setattr(sys.modules["apyib"], name, mod)
        mods[name] = sys.modules[full]
    return types.SimpleNamespace(**mods)
