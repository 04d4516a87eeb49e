"""Run one complex GEMM of a given shape twice (for ncu).

    python -m apyib_gb300.profile_gemm M N K [tf32x3|df64|fp64]

A: [M,K] complex128 row-major, B: [N,K] (used transposed), random normal.
"""
import ctypes
import sys

import torch

from . import _lib
from .device import ptr, stream_ptr, workspace


def main(argv):
    M, N, K = (int(a) for a in argv[:3])
    kind = argv[3] if len(argv) > 3 else "tf32x3"
    torch.cuda.set_device(0)
    A = torch.randn(M, K, dtype=torch.complex128, device="cuda")
    B = torch.randn(N, K, dtype=torch.complex128, device="cuda")
    C = torch.zeros(M, N, dtype=torch.complex128, device="cuda")
    if kind == "tf32x3":
        nb = _lib.load().agb_cgemm_tf32x3_scratch_bytes(M, N, K)
        buf, sp, _ = workspace(nb)
        buf.zero_()
    elif kind == "df64":
        nb = _lib.load().agb_zgemm_df64_scratch_bytes(M, N, K)
        buf, sp, _ = workspace(nb)
    for _ in range(2):
        if kind == "tf32x3":
            _lib.call("agb_cgemm_tf32x3", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
        elif kind == "df64":
            _lib.call("agb_zgemm_df64_ex", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
        else:
            _lib.call("agb_zgemm", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      stream_ptr())
    if kind == "tf32x3":
        _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
    torch.cuda.synchronize()
    print("ok", kind, M, N, K)


if __name__ == "__main__":
    main(sys.argv[1:])
