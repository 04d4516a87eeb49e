"""Run the J/K Fock build on nbf basis functions a few times (for timing and ncu).

    python -m apyib_gb300.profile_jk [nbf] [repeats] [sym|sym64|general]

Real symmetric AO integrals (mn|ls) = sum_L A_Lmn A_Lls from seeded random
symmetric factors (made exactly symmetric in (l, s)), a complex Hermitian density;
runs the double-float kernel that reads the l <= s half (sym, default), its FP64
twin (sym64) or the general double-float kernel, and prints the mean time (CUDA
events on the launch stream) and the bandwidth the result's full tensor
(8 nbf^4 B) would need.
"""
import sys

import torch

from .linalg import jk_fock


def main(argv):
    n = int(argv[0]) if argv else 150
    reps = int(argv[1]) if len(argv) > 1 else 5
    torch.cuda.set_device(0)
    g = torch.Generator(device="cpu").manual_seed(0)
    A = torch.randn(3 * n, n, n, generator=g, dtype=torch.float64)
    A = ((A + A.transpose(1, 2)) / (2 * (3 * n * n) ** 0.5)).cuda()
    eri = torch.einsum("Lmn,Lls->mnls", A, A)
    del A
    eri = (0.5 * (eri + eri.transpose(2, 3))).contiguous()
    kind = argv[2] if len(argv) > 2 else "sym"
    if kind == "general":
        eri[0, 0, 0, 1] = eri[0, 0, 0, 1] * (1 + 2.0 ** -40) + 1e-300   # not (l, s)-symmetric: general kernel
    C = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.complex128))[0].cuda()
    D = (C[:, : n // 4] @ C[:, : n // 4].conj().T).contiguous()
    h = torch.zeros(n, n, dtype=torch.complex128, device="cuda")
    prec = "fp64" if kind == "sym64" else "df64"
    jk_fock(eri, D, h, 1.0, precision=prec)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        jk_fock(eri, D, h, 1.0, precision=prec)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    print(f"jk_fock ({kind}) nbf={n}: {ms:.3f} ms per call, {8.0 * n ** 4 / ms / 1e6:.1f} GB/s of ERI")


if __name__ == "__main__":
    main(sys.argv[1:])
