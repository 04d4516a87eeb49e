"""ctypes binding of ``libapyib_gb300.so`` (declared in include/apyib_gb300.h).

The library is built in-tree by ``apyib_gb300.build``.  There is no CPU
fallback: every public entry point of this package raises when the library
is missing or a CUDA device is not available.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None

AGB_OK = 0
AGB_ERR_ARG = 1
AGB_ERR_CUDA = 2
AGB_ERR_UNSUPPORTED = 3
AGB_ERR_TIMEOUT = 4
AGB_ERR_WORKSPACE = 5

PREC_FP64 = 0
PREC_TF32X3 = 1
PREC_DF64 = 2
PREC_OZAKI = 3

PLAN_MIXED = 1
PLAN_NO_SINGLES = 2
PLAN_MP2 = 4

RES_CONST = 1
RES_ETERM = 2

OEI_OVERLAP, OEI_KINETIC, OEI_POTENTIAL, OEI_DIPOLE, OEI_NABLA, OEI_ANGMOM, OEI_OVERLAP_HALF = range(7)
AO_ROW_MAX = 16            # coefficients per row of agb_ao_transform_axis

_c = ctypes
_vp = _c.c_void_p
_i64 = _c.c_int64
_d = _c.c_double
_int = _c.c_int
_sz = _c.c_size_t



class Basis(_c.Structure):
    """agb_basis: a contracted Gaussian basis, every array a device pointer."""
    _fields_ = [("natom", _int), ("nshell", _int), ("ncart", _int), ("lmax", _int),
                ("atom_xyz", _vp), ("atom_charge", _vp), ("shell_l", _vp), ("shell_atom", _vp),
                ("shell_nprim", _vp), ("shell_prim0", _vp), ("shell_cart0", _vp), ("bf_shell", _vp),
                ("exps", _vp), ("coefs", _vp)]


# name -> (restype, argtypes)
SIGNATURES = {
    "agb_version": (_int, []),
    "agb_launch_count": (_c.c_ulonglong, []),
    "agb_last_error": (_c.c_char_p, []),
    "agb_zgemm": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d, _vp, _i64,
                         _vp]),
    "agb_zgemm_scratch_bytes": (_sz, [_i64, _i64, _i64]),
    "agb_zgemm_ex": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d, _vp,
                            _i64, _vp, _sz, _vp]),
    "agb_zgemm_df64": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d, _vp,
                              _i64, _vp]),
    "agb_zgemm_df64_scratch_bytes": (_sz, [_i64, _i64, _i64]),
    "agb_zgemm_df64_ex": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d,
                                 _vp, _i64, _vp, _sz, _vp]),
    "agb_zgemm_oz_scratch_bytes": (_sz, [_i64, _i64, _i64]),
    "agb_zgemm_oz": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d, _vp,
                            _i64, _vp, _sz, _vp]),
    "agb_cgemm_tf32x3_scratch_bytes": (_sz, [_i64, _i64, _i64]),
    "agb_cgemm_tf32x3": (_int, [_i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _int, _vp, _i64, _i64, _int, _d, _d, _vp,
                                _i64, _vp, _sz, _vp]),
    "agb_scratch_status": (_int, [_vp, _vp]),
    "agb_zgemm_batched": (_int, [_i64, _i64, _i64, _i64, _d, _d, _vp, _i64, _i64, _i64, _int, _vp, _i64, _i64, _i64,
                                 _int, _d, _d, _vp, _i64, _i64, _vp]),
    "agb_zdet_inv_batched": (_int, [_i64, _int, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _vp]),
    "agb_cisd_plan_gemm_timing": (_int, [_vp, _int]),
    "agb_cisd_plan_gemm_timing_collect": (_int, [_vp, _d, _c.POINTER(_int), _c.POINTER(_d), _c.POINTER(_d)]),
    "agb_compute_f_so": (_int, [_vp, _i64, _vp, _vp]),
    "agb_compute_eri_so": (_int, [_vp, _i64, _i64, _i64, _i64, _vp, _vp]),
    "agb_cisd_plan_create": (_int, [_int, _int, _int, _c.POINTER(_vp)]),
    "agb_cisd_plan_destroy": (_int, [_vp]),
    "agb_cisd_plan_workspace_bytes": (_int, [_vp, _c.POINTER(_sz)]),
    "agb_cisd_plan_set_workspace": (_int, [_vp, _vp, _sz]),
    "agb_cisd_plan_sizes": (_int, [_vp, _c.POINTER(_i64), _c.POINTER(_i64)]),
    "agb_cisd_set_fock": (_int, [_vp, _vp, _vp, _vp]),
    "agb_cisd_blocks_from_mo": (_int, [_vp, _vp, _vp]),
    "agb_cisd_blocks_from_so": (_int, [_vp, _vp, _vp]),
    "agb_cisd_factor_scratch_bytes": (_sz, [_vp, _i64]),
    "agb_cisd_blocks_from_factors": (_int, [_vp, _vp, _i64, _vp, _sz, _int, _vp]),
    "agb_cisd_residual": (_int, [_vp, _int, _vp, _d, _d, _int, _vp, _vp]),
    "agb_cisd_status": (_int, [_vp, _vp]),
    "agb_cisd_update": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "agb_vec_dots": (_int, [_i64, _i64, _d, _d, _vp, _c.POINTER(_vp), _int, _vp, _vp, _sz, _vp]),
    "agb_vec_partials_bytes": (_sz, [_int]),
    "agb_vec_dots_noalloc": (_int, [_i64, _i64, _d, _d, _vp, _c.POINTER(_vp), _int, _vp, _vp]),
    "agb_cisd_combine": (_int, [_vp, _c.POINTER(_vp), _c.POINTER(_d), _int, _vp, _vp, _vp, _vp, _sz, _vp]),
    "agb_cisd_unpack": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "agb_cisd_pack": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "agb_cisd_guess": (_int, [_vp, _vp, _vp]),
    "agb_mp2_so": (_int, [_vp, _vp, _vp, _vp, _sz, _vp]),
    "agb_mp2_spatial": (_int, [_vp, _i64, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "agb_ao2mo_scratch_bytes": (_sz, [_i64, _i64, _int]),
    "agb_ao2mo": (_int, [_vp, _i64, _vp, _i64, _vp, _vp, _sz, _int, _vp]),
    "agb_jk_fock_scratch_bytes": (_sz, [_i64]),
    "agb_jk_fock": (_int, [_vp, _i64, _vp, _vp, _d, _vp, _vp, _sz, _vp]),
    "agb_jk_fock_sym": (_int, [_vp, _i64, _vp, _vp, _d, _vp, _vp, _sz, _vp]),
    "agb_jk_fock_sym64": (_int, [_vp, _i64, _vp, _vp, _d, _vp, _vp, _sz, _vp]),
    "agb_ao_one_electron": (_int, [_c.POINTER(Basis), _int, _c.POINTER(_d), _vp, _vp]),
    "agb_ao_eri": (_int, [_c.POINTER(Basis), _vp, _vp]),
    "agb_ao_one_electron_deriv": (_int, [_c.POINTER(Basis), _int, _vp, _vp]),
    "agb_ao_eri_deriv": (_int, [_c.POINTER(Basis), _vp, _vp]),
    "agb_ao_transform_axis": (_int, [_vp, _i64, _int, _i64, _int, _vp, _vp, _vp, _vp, _vp]),
}


class AGBError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"apyib_gb300 error {status}: {msg}")
        self.status = status


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the shared library (building it in place first if it is missing
    and nvcc is available)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} is not built; run apyib_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status):
    if status != AGB_OK:
        msg = load().agb_last_error()
        raise AGBError(status, msg.decode() if msg else "")


def call(name, *args):
    check(getattr(load(), name)(*args))
