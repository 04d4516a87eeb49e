"""Batched small complex linear algebra of the library (agb_zgemm_batched,
agb_zdet_inv_batched) against torch's FP64 complex matmul / linalg on the same
matrices: broadcast batch operands, strided and conjugated views, pivoting (a zero
leading element), n = 1 and the largest supported n = 96, and a singular matrix
reported through info."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402
from apyib_gb300.linalg import bdet_inv, bdot, bmm  # noqa: E402


def crand(g, *shape):
    return torch.randn(*shape, dtype=torch.complex128, device="cuda", generator=g)


@pytest.mark.parametrize("nb,M,N,K", [(7, 10, 38, 10), (1, 33, 65, 17), (40, 1, 1, 1444), (3, 96, 96, 96)])
def test_batched_products_match_torch(nb, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(nb * 1000 + M)
    A = crand(g, nb, M, K)
    B = crand(g, 1, K, N)                              # broadcast along the batch
    np.testing.assert_allclose(bmm(A, B).cpu().numpy(), (A @ B).cpu().numpy(), rtol=0, atol=1e-12 * K)
    Bt = crand(g, nb, N, K)
    ref = A.conj() @ Bt.transpose(1, 2)
    got = bmm(A, Bt, conjA=True, transB=True)
    np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=0, atol=1e-12 * K)
    At = A.transpose(1, 2)                             # a strided view, used transposed
    B2 = crand(g, nb, K, N)
    got = bmm(At, B2, transA=True, conjB=True, alpha=0.5 - 0.25j)
    np.testing.assert_allclose(got.cpu().numpy(), ((0.5 - 0.25j) * (A @ B2.conj())).cpu().numpy(), rtol=0,
                               atol=1e-12 * K)
    X, Y = crand(g, nb, M, K), crand(g, 1, M, K)
    np.testing.assert_allclose(bdot(X, Y).cpu().numpy(), (X * Y).sum((1, 2)).cpu().numpy(), rtol=0,
                               atol=1e-12 * M * K)


@pytest.mark.parametrize("n", [1, 2, 10, 37, 96])
def test_det_inverse_match_torch(n):
    g = torch.Generator(device="cuda").manual_seed(n)
    S = crand(g, 5, n, n) + 2.0 * torch.eye(n, dtype=torch.complex128, device="cuda")
    if n > 1:
        S[1, 0, 0] = 0.0                               # the first step must pivot
        S[2] = S[2][torch.randperm(n, device="cuda", generator=g)]
    det, inv = bdet_inv(S)
    ref_det = torch.linalg.det(S)
    ref_inv = torch.linalg.inv(S)
    np.testing.assert_allclose(det.cpu().numpy(), ref_det.cpu().numpy(), rtol=1e-11, atol=0)
    np.testing.assert_allclose(inv.cpu().numpy(), ref_inv.cpu().numpy(), rtol=0,
                               atol=1e-11 * float(ref_inv.abs().max()))
    eye = torch.eye(n, dtype=torch.complex128, device="cuda").expand(5, n, n)
    assert float((S @ inv - eye).abs().max()) < 1e-11


def test_singular_matrix_is_reported():
    S = torch.zeros((2, 3, 3), dtype=torch.complex128, device="cuda")
    S[0] = torch.eye(3)
    S[1, 0] = torch.tensor([1.0, 2.0, 3.0])
    S[1, 1] = 2.0 * S[1, 0]                            # rank deficient
    S[1, 2, 2] = 1.0
    with pytest.raises(ZeroDivisionError):
        bdet_inv(S)
    with pytest.raises(_lib.AGBError):
        bdet_inv(torch.zeros((1, 97, 97), dtype=torch.complex128, device="cuda"))
