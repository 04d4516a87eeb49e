"""Run one complex GEMM of a given shape twice (for ncu).

    python -m apyib_gb300.profile_gemm M N K [tf32x3|df64|oz|fp64]

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
    elif kind == "oz":
        nb = _lib.load().agb_zgemm_oz_scratch_bytes(M, N, K)
        buf, sp, _ = workspace(nb)
        buf[:256].zero_()

    def run():
        if kind == "tf32x3":
            _lib.call("agb_cgemm_tf32x3", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
        elif kind == "df64":
            _lib.call("agb_zgemm_df64_ex", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
        elif kind == "oz":
            _lib.call("agb_zgemm_oz", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
        else:
            _lib.call("agb_zgemm", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                      stream_ptr())

    for _ in range(2):
        run()
    if kind in ("tf32x3", "oz"):
        _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    print("ok", kind, M, N, K, f"{ms:.3f} ms", f"{8.0 * M * N * K / ms / 1e9:.1f} TFLOP/s (8MNK)")


if __name__ == "__main__":
    main(sys.argv[1:])
