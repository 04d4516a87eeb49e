"""GPU parity of the library kernels against NumPy (complex128)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402
from apyib_gb300.device import ptr, stream_ptr, to_dev, workspace  # noqa: E402
from apyib_gb300.linalg import jk_fock, zmm  # noqa: E402
from oracle import port  # noqa: E402
from tests.gpu_util import crandn  # noqa: E402


@pytest.mark.parametrize("M,N,K,ta,tb,ca,cb", [
    (1, 1, 1, False, False, False, False),
    (37, 53, 29, False, False, False, False),
    (64, 64, 64, True, False, True, False),
    (130, 70, 300, False, True, False, True),
    (5, 7, 5000, True, True, True, True),      # split-K would apply with scratch
])
def test_zgemm_matches_numpy(M, N, K, ta, tb, ca, cb):
    rng = np.random.default_rng(M * 7 + N)
    A = crandn(rng, *((K, M) if ta else (M, K)))
    B = crandn(rng, *((N, K) if tb else (K, N)))
    opA = A.T if ta else A
    opB = B.T if tb else B
    if ca:
        opA = opA.conj()
    if cb:
        opB = opB.conj()
    ref = (2 - 1j) * opA @ opB
    C = zmm(to_dev(A), to_dev(B), transA=ta, conjA=ca, transB=tb, conjB=cb, alpha=2 - 1j).cpu().numpy()
    np.testing.assert_allclose(C, ref, rtol=0, atol=1e-12 * np.sqrt(K) * 4)


def tf32_gemm(A, B, alpha=1.0, beta=0.0, C=None, transB=False):
    Ad, Bd = to_dev(A), to_dev(B)
    M, K = A.shape
    N = B.shape[0] if transB else B.shape[1]
    out = to_dev(C) if C is not None else torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    nb = _lib.load().agb_cgemm_tf32x3_scratch_bytes(M, N, K)
    buf, sp, _ = workspace(nb)
    torch.cuda.synchronize()
    buf.zero_()
    sBk, sBn = (1, K) if transB else (N, 1)
    a, b = complex(alpha), complex(beta)
    _lib.call("agb_cgemm_tf32x3", M, N, K, a.real, a.imag, ptr(Ad), K, 1, 0, ptr(Bd), sBk, sBn, 0, b.real, b.imag,
              ptr(out), N, ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
    _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
    return out.cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(128, 128, 16), (1, 1, 1), (200, 300, 77), (60, 240, 6000), (513, 129, 1000),
                                   (2000, 60, 240), (240, 60, 60000), (300, 64, 500), (100, 65, 100), (33, 17, 100),
                                   (64, 64, 64), (1100, 1030, 500), (1024, 2049, 64)])
def test_tf32x3_gemm_accuracy(M, N, K):
    """3xTF32 complex GEMM: error ~1e-6 relative to sum|a||b| (FP32-level).  N <= 64 takes
    the 64-wide tile (split over K for (240, 60, 60000)); M <= 64 an A operand whose
    64-row planes the 128-row tile reads past; both extents >= 1024 the CTA-pair kernel
    (ragged pair tiles in (1100, 1030, 500))."""
    rng = np.random.default_rng(M + N + K)
    A = crandn(rng, M, K)
    B = crandn(rng, K, N)
    ref = A @ B
    got = tf32_gemm(A, B)
    scale = np.abs(A) @ np.abs(B)
    err = np.abs(got - ref) / scale
    assert err.max() < 2e-6, err.max()


def test_tf32x3_gemm_alpha_beta_and_transposed_b():
    rng = np.random.default_rng(5)
    A = crandn(rng, 150, 90)
    Bt = crandn(rng, 170, 90)
    C0 = crandn(rng, 150, 170)
    ref = (0.5 + 2j) * A @ Bt.T + (1 - 1j) * C0
    got = tf32_gemm(A, Bt, alpha=0.5 + 2j, beta=1 - 1j, C=C0, transB=True)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5
    # the same on the 64-wide tile
    Bn, Cn = Bt[:40], C0[:, :40]
    ref = (0.5 + 2j) * A @ Bn.T + (1 - 1j) * Cn
    got = tf32_gemm(A, Bn, alpha=0.5 + 2j, beta=1 - 1j, C=Cn, transB=True)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5


@pytest.mark.parametrize("n,symmetric", [(1, True), (2, True), (19, True), (33, True), (45, True), (70, True),
                                         (33, False)])
def test_jk_fock_matches_oracle(n, symmetric):
    """Double-float J/K against the FP64 NumPy restatement; n = 45, 70 leave a ragged
    last block of rows, n = 33 a ragged last lane round.  ERIs symmetric in (l, s) take
    the half-reading kernel (checked against the general one too); the non-symmetric
    case checks that no integral symmetry is assumed otherwise."""
    import ctypes

    from apyib_gb300 import _lib
    from apyib_gb300.device import ptr, stream_ptr, workspace
    from apyib_gb300.linalg import last_pair_symmetric
    rng = np.random.default_rng(3 + n)
    if symmetric:
        A = rng.standard_normal((40, n, n))
        A = A + A.transpose(0, 2, 1)
        eri = np.einsum("Lmn,Lls->mnls", A, A) / 40
        eri = 0.5 * (eri + eri.transpose(0, 1, 3, 2))      # exactly symmetric in (l, s)
    else:
        eri = rng.standard_normal((n, n, n, n))
    D = crandn(rng, n, n)
    h = crandn(rng, n, n)
    eri_d = to_dev(eri, torch.float64)
    assert last_pair_symmetric(eri_d) == symmetric
    ref = port.jk_fock(h, eri, D, 0.5)
    scale = np.abs(eri).max() * np.abs(D).max() * n * n
    for prec, tol in (("fp64", 1e-14), ("df64", 1e-13)):
        F = jk_fock(eri_d, to_dev(D), to_dev(h), 0.5, precision=prec).cpu().numpy()
        np.testing.assert_allclose(F, ref, atol=(tol if symmetric else 1e-13) * scale)
        F2 = jk_fock(eri_d, to_dev(D), to_dev(h), 0.5, precision=prec).cpu().numpy()
        np.testing.assert_array_equal(F, F2)    # deterministic
    if symmetric:                               # the general kernel on the same input
        Fg = torch.empty((n, n), dtype=torch.complex128, device="cuda")
        nb = _lib.load().agb_jk_fock_scratch_bytes(n)
        buf, sp, _ = workspace(nb)
        Dd, hd = to_dev(D), to_dev(h)            # held: the pointers must stay valid
        _lib.call("agb_jk_fock", ptr(eri_d), n, ptr(Dd), ptr(hd), 0.5, ptr(Fg), ctypes.c_void_p(sp),
                  ctypes.c_size_t(nb), stream_ptr())
        np.testing.assert_allclose(F, Fg.cpu().numpy(), atol=1e-13 * scale)


def test_so_expansion_matches_oracle():
    from apyib_gb300 import utils
    rng = np.random.default_rng(4)
    F = crandn(rng, 5, 5)
    g = crandn(rng, 3, 4, 5, 2)
    np.testing.assert_array_equal(utils.compute_F_SO(None, F), port.compute_F_SO(F))
    np.testing.assert_array_equal(utils.compute_ERI_SO(None, g), port.compute_ERI_SO(g))


@pytest.mark.parametrize("M,N,K", [(37, 53, 29), (130, 70, 3000), (5, 7, 20000)])
def test_df64_gemm_accuracy(M, N, K):
    """Double-float GEMM: error ~1e-13 relative to sum|a||b| (vs ~1e-16 FP64, ~1e-6 3xTF32)."""
    rng = np.random.default_rng(M * 3 + K)
    A = crandn(rng, M, K)
    B = crandn(rng, K, N)
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    _lib.call("agb_zgemm_df64", M, N, K, 1.0, 0.0, ptr(Ad), K, 1, 0, ptr(Bd), N, 1, 0, 0.0, 0.0, ptr(C), N,
              stream_ptr())
    got = C.cpu().numpy()
    ref = A @ B
    err = np.abs(got - ref) / (np.abs(A) @ np.abs(B))
    assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("M,N,K", [(37, 53, 29), (300, 200, 5000), (5, 7, 20000)])
def test_df64_gemm_presplit_3m_accuracy(M, N, K):
    """The pre-split three-product double-float path keeps ~1e-13 relative accuracy."""
    rng = np.random.default_rng(M * 5 + K)
    A = crandn(rng, M, K)
    B = crandn(rng, K, N)
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    nb = _lib.load().agb_zgemm_df64_scratch_bytes(M, N, K)
    buf, sp, _ = workspace(nb)
    _lib.call("agb_zgemm_df64_ex", M, N, K, 1.0, 0.0, ptr(Ad), K, 1, 0, ptr(Bd), N, 1, 0, 0.0, 0.0, ptr(C), N,
              ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
    got = C.cpu().numpy()
    ref = A @ B
    err = np.abs(got - ref) / (np.abs(A) @ np.abs(B))
    assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("ny,n1,n2,w1,w2", [(3, 50, 7000, 1.0, 4.0), (7, 0, 100000, 1.0, 4.0),
                                            (12, 1234, 54321, 0.3, 2.5), (1, 9, 0, 2.0, 1.0)])
def test_vec_dots_matches_numpy(ny, n1, n2, w1, w2):
    """DIIS Gram row (double-float products and sums) against NumPy: ~1e-14 of sum |x||y|."""
    rng = np.random.default_rng(ny + n1)
    n = n1 + n2
    x = crandn(rng, n)
    ys = [crandn(rng, n) for _ in range(ny)]
    xd = to_dev(x)
    yd = [to_dev(y) for y in ys]
    arr = (ctypes.c_void_p * ny)(*[y.data_ptr() for y in yd])
    out = torch.zeros(16, dtype=torch.complex128, device="cuda")
    nb = _lib.load().agb_vec_partials_bytes(ny)
    buf, sp, _ = workspace(nb)
    _lib.call("agb_vec_dots", n1, n2, w1, w2, ptr(xd), arr, ny, ptr(out), ctypes.c_void_p(sp), ctypes.c_size_t(nb),
              stream_ptr())
    got = out[:ny].cpu().numpy()
    w = np.concatenate([np.full(n1, w1), np.full(n2, w2)])
    ref = np.array([np.sum(w * y.conj() * x) for y in ys])
    bound = np.array([np.sum(w * np.abs(y) * np.abs(x)) for y in ys])
    assert np.all(np.abs(got - ref) <= 1e-13 * bound), np.abs(got - ref) / bound
