"""Ozaki-split bf16 tensor-core GEMM (agb_zgemm_oz): FP64-level accuracy against
NumPy complex128 products on both of its kernels (K <= 1024: the one-pass 4M kernel,
256-long exact chunks; longer K: the three-pass 3M kernel, 512-long chunks),
including K crossing the exact chunks,
ragged tiles, strided / conjugated operands, alpha/beta, rows of very different
scale, integer data whose products must come out exact, and the base residual
of the mixed solver.  Tolerance: 3e-12 of sum |a||b| per element (42-bit slices
of each row relative to the row's largest entry; the 3M imaginary part
P3 - P1 - P2 about doubles the absolute error)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402
from apyib_gb300.device import ptr, stream_ptr, to_dev, workspace  # noqa: E402
from tests.gpu_util import crandn  # noqa: E402

TOL = 3e-12


def oz(A, B, alpha=1.0, beta=0.0, C=None, conjA=False, conjB=False, transA=False, transB=False, extra=1):
    """op(A) op(B) through agb_zgemm_oz; op = transpose / conjugate flags like agb_zgemm.
    extra > 1 multiplies the scratch, which lets the GEMM slice A once for all products."""
    Ad, Bd = to_dev(A), to_dev(B)
    M, K = (A.shape[1], A.shape[0]) if transA else A.shape
    N = B.shape[0] if transB else B.shape[1]
    sAm, sAk = (1, M) if transA else (K, 1)
    sBk, sBn = (1, K) if transB else (N, 1)
    Cd = to_dev(C) if C is not None else torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    nb = _lib.load().agb_zgemm_oz_scratch_bytes(M, N, K) * extra
    buf, sp, _ = workspace(nb)
    buf[:256].zero_()
    alpha, beta = complex(alpha), complex(beta)
    _lib.call("agb_zgemm_oz", M, N, K, alpha.real, alpha.imag, ptr(Ad), sAm, sAk, int(conjA), ptr(Bd), sBk, sBn,
              int(conjB), beta.real, beta.imag, ptr(Cd), N, ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
    _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
    return Cd.cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (130, 260, 700), (300, 129, 20), (256, 384, 1500),
                                   (5, 7, 3), (200, 160, 1025), (129, 33, 1024), (257, 31, 257), (64, 96, 96),
                                   # several tiles per persistent CTA; last column tiles 16 or 32 wide;
                                   # one to four 256-long chunks per tile
                                   (20000, 150, 150), (3000, 100, 300), (2000, 20, 520), (1500, 64, 1024),
                                   # the largest K sliced in one read (32 rows x 192 k staged) and the next
                                   (3000, 70, 192), (3000, 70, 193)])
def test_oz_gemm_accuracy(M, N, K):
    rng = np.random.default_rng(M + 7 * N + 13 * K)
    A = crandn(rng, M, K)
    B = crandn(rng, K, N)
    got = oz(A, B)
    ref = A @ B
    err = np.abs(got - ref) / (np.abs(A) @ np.abs(B))
    assert err.max() < TOL, err.max()


def test_oz_gemm_strides_conj_alpha_beta():
    rng = np.random.default_rng(5)
    M, N, K = 140, 150, 600
    A = crandn(rng, K, M)          # used transposed and conjugated
    B = crandn(rng, N, K)          # used transposed
    C0 = crandn(rng, M, N)
    alpha, beta = 0.7 - 1.3j, -0.4 + 0.25j
    got = oz(A, B, alpha=alpha, beta=beta, C=C0, conjA=True, transA=True, transB=True)
    ref = alpha * (A.T.conj() @ B.T) + beta * C0
    bound = abs(alpha) * (np.abs(A.T) @ np.abs(B.T)) + abs(beta) * np.abs(C0)
    assert (np.abs(got - ref) / bound).max() < TOL


def test_oz_gemm_row_scales():
    """Rows and columns spanning 12 decades keep accuracy relative to their own scale."""
    rng = np.random.default_rng(9)
    M, N, K = 160, 150, 900
    A = crandn(rng, M, K) * np.logspace(-6, 6, M)[:, None]
    B = crandn(rng, K, N) * np.logspace(4, -4, N)[None, :]
    got = oz(A, B)
    ref = A @ B
    err = np.abs(got - ref) / (np.abs(A) @ np.abs(B))
    assert err.max() < TOL, err.max()


def test_oz_gemm_extreme_exponents():
    """Row and column scales from 2^-520 to 2^505: outputs from subnormal (2^-1040) to
    2^505 times O(1) go through the epilogue's integer conversion to FP64 and its
    fallback for results outside the normal range."""
    rng = np.random.default_rng(13)
    M, N, K = 96, 48, 100
    Au, Bu = crandn(rng, M, K), crandn(rng, K, N)
    rs = np.array([2.0 ** -520, 1.0, 2.0 ** 505])[np.arange(M) % 3]
    cs = np.array([2.0 ** -520, 1.0])[np.arange(N) % 2]
    got = oz(Au * rs[:, None], Bu * cs[None, :])
    scale = rs[:, None] * cs[None, :]
    ref = (Au @ Bu) * scale
    bound = (np.abs(Au) @ np.abs(Bu)) * scale
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - ref) <= TOL * bound + 2.0 ** -1072)


@pytest.mark.parametrize("conjA", [False, True])
def test_oz_gemm_single_slicing_pass_is_identical(conjA):
    """With room for all three parts' A slices the GEMM slices A in one pass: the same
    slices and products, so the same bits as part-by-part slicing."""
    rng = np.random.default_rng(17)
    A, B, C0 = crandn(rng, 300, 1100), crandn(rng, 1100, 130), crandn(rng, 300, 130)
    one = oz(A, B, alpha=0.3 + 1j, beta=0.5, C=C0, conjA=conjA)
    fused = oz(A, B, alpha=0.3 + 1j, beta=0.5, C=C0, conjA=conjA, extra=4)
    np.testing.assert_array_equal(one, fused)


@pytest.mark.parametrize("M,N,K", [(3000, 150, 150), (700, 40, 600)])
def test_oz_gemm_transposed_operands_are_identical(M, N, K):
    """Short K: operands read along k or along rows (the slicer's two transposed tile loads)
    give the same slices in the K-blocked layout, so the same bits."""
    rng = np.random.default_rng(19)
    A, B = crandn(rng, M, K), crandn(rng, K, N)
    kfast = oz(A, B.T.copy(), transB=True)                    # A: k-fast rows; B: k-fast columns
    rowfast = oz(A.T.copy(), B, transA=True)                  # A: adjacent rows; B: adjacent columns
    np.testing.assert_array_equal(kfast, rowfast)
    err = np.abs(rowfast - A @ B) / (np.abs(A) @ np.abs(B))
    assert err.max() < TOL, err.max()


@pytest.mark.parametrize("K", [2048, 1000])
def test_oz_gemm_integer_products_exact(K):
    """Small-integer operands have exact slices, so every partial sum is an exact
    integer: any rounding inside the tensor-core accumulation would show (K = 1000:
    four 256-long chunks of the one-pass kernel, two products per accumulator)."""
    rng = np.random.default_rng(11)
    M, N = 256, 256
    A = rng.integers(-127, 128, (M, K)) + 1j * rng.integers(-127, 128, (M, K))
    B = rng.integers(-127, 128, (K, N)) + 1j * rng.integers(-127, 128, (K, N))
    got = oz(A.astype(np.complex128), B.astype(np.complex128))
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    np.testing.assert_array_equal(got, ref)


def test_oz_rejects_small_scratch():
    A = to_dev(np.ones((4, 4), dtype=complex))
    C = torch.zeros((4, 4), dtype=torch.complex128, device="cuda")
    buf, sp, _ = workspace(1024)
    st = _lib.load().agb_zgemm_oz(4, 4, 4, 1.0, 0.0, ptr(A), 4, 1, 0, ptr(A), 4, 1, 0, 0.0, 0.0, ptr(C), 4,
                                  ctypes.c_void_p(sp), ctypes.c_size_t(1024), stream_ptr())
    assert st == _lib.AGB_ERR_WORKSPACE


def test_oz_base_residual_matches_fp64():
    """The mixed plan's residual with Ozaki GEMMs (the ring GEMM at o/v = 20/80 has
    enough tiles to take the tensor-core path) against the FP64 residual."""
    from apyib_gb300 import synthetic
    from apyib_gb300.cisd import CISDPlan
    prob = synthetic.so_factors(20, 80, seed=2)
    eps = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan = CISDPlan(20, 80, mixed=True)
    plan.set_fock(torch.as_tensor(prob.fock_so()), eps)
    plan.blocks_from_factors(torch.as_tensor(prob.B), precision=_lib.PREC_OZAKI)
    t = plan.guess()
    r64 = plan.residual(t, -0.1, _lib.PREC_FP64)
    roz = plan.residual(t, -0.1, _lib.PREC_OZAKI)
    plan.check_status()
    scale = r64.abs().max().item()
    assert (roz - r64).abs().max().item() < 1e-11 * max(scale, 1.0)
    # blocks built with FP64 factor products give the same residual
    plan2 = CISDPlan(20, 80, mixed=True)
    plan2.set_fock(torch.as_tensor(prob.fock_so()), eps)
    plan2.blocks_from_factors(torch.as_tensor(prob.B), precision=_lib.PREC_FP64)
    r2 = plan2.residual(t, -0.1, _lib.PREC_FP64)
    assert (r2 - r64).abs().max().item() < 1e-11 * max(scale, 1.0)
