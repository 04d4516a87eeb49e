"""CPU-side checks of the C-ABI library: it builds, loads and exports every
entry point declared in include/apyib_gb300.h (no compute calls)."""
import ctypes
import os
import re

import pytest

from apyib_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "apyib_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_loads():
    build.build()
    lib = _lib.load()
    assert lib.agb_version() >= 100


def test_every_declared_symbol_is_exported_and_bound():
    lib = ctypes.CDLL(_lib.lib_path())
    syms = declared_symbols()
    assert len(syms) > 20
    for s in syms:
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_no_unknown_bindings():
    syms = set(declared_symbols())
    assert set(_lib.SIGNATURES) <= syms


def test_plan_sizes_without_gpu():
    """Plan creation and workspace sizing are host-only."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.call("agb_cisd_plan_create", 60, 240, 0, ctypes.byref(h))
    nb = ctypes.c_size_t()
    _lib.call("agb_cisd_plan_workspace_bytes", h, ctypes.byref(nb))
    n1, n2 = ctypes.c_int64(), ctypes.c_int64()
    _lib.call("agb_cisd_plan_sizes", h, ctypes.byref(n1), ctypes.byref(n2))
    assert n1.value == 60 * 240 and n2.value == (60 * 59 // 2) * (240 * 239 // 2)
    assert 30e9 < nb.value < 200e9
    lib.agb_cisd_plan_destroy(h)


def test_bad_arguments_are_rejected():
    h = ctypes.c_void_p()
    with pytest.raises(_lib.AGBError):
        _lib.call("agb_cisd_plan_create", 3, 4, 0, ctypes.byref(h))   # odd o
    with pytest.raises(_lib.AGBError):
        _lib.call("agb_cisd_plan_set_workspace", ctypes.c_void_p(0), ctypes.c_void_p(0), 0)


@pytest.mark.parametrize("entry,extra", [("agb_zgemm", []), ("agb_zgemm_df64", []),
                                         ("agb_zgemm_ex", [ctypes.c_void_p(0), ctypes.c_size_t(0)]),
                                         ("agb_zgemm_df64_ex", [ctypes.c_void_p(0), ctypes.c_size_t(0)]),
                                         ("agb_zgemm_oz", [ctypes.c_void_p(0), ctypes.c_size_t(0)]),
                                         ("agb_cgemm_tf32x3", [ctypes.c_void_p(0), ctypes.c_size_t(0)])])
def test_gemm_rejects_short_leading_dimension(entry, extra):
    """A row-major C needs ldc >= N (fewer would overlap its rows and write past the
    buffer): every GEMM entry point refuses it before touching the device."""
    fake = ctypes.c_void_p(4096)          # never dereferenced: the call returns first
    M, N, K = 8, 6, 4
    with pytest.raises(_lib.AGBError, match="ldc"):
        _lib.call(entry, M, N, K, 1.0, 0.0, fake, K, 1, 0, fake, N, 1, 0, 0.0, 0.0, fake, N - 1, *extra,
                  ctypes.c_void_p(0))
