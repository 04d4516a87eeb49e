"""apyib_gb300: GB300-native (sm_103a) correlated-wavefunction hot path of apyib.

Drop-in classes mirroring the reference interface:
  Hamiltonian, hf_wfn, mp2_wfn, ci_wfn and the utils helpers.
All heavy contractions run in hand-written CUDA kernels of the in-tree
library libapyib_gb300.so (C ABI in include/apyib_gb300.h).
"""
from . import build  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # Lazy imports keep `import apyib_gb300` cheap and torch-free until used.
    import importlib
    if name in ("hf_wfn", "mp2_wfn", "ci_wfn", "utils", "hamiltonian", "cisd", "synthetic", "adjoint"):
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
