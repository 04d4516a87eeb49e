"""The closed-shell CISD / CID engine (apyib_gb300.spatial.SpatialCISD: the reference's
spatial residual as library GEMMs) with that GEMM pointed at torch on the CPU: its
residual must equal the oracle's restatement of apyib/ci_wfn.py:458-490 term for term,
and with t1 = 0 the reference's symmetrised CID residual (:84-95), on random complex
amplitudes and a non-diagonal complex Fock matrix; its solve must reproduce the
closed-shell energies the spin-orbital oracle gives (alpha-beta amplitude block)."""
import numpy as np
import pytest
import torch

from apyib_gb300 import spatial
from oracle import port


@pytest.fixture
def torch_gemm(monkeypatch):
    def zmm(A, B, transA=False, conjA=False, transB=False, conjB=False, alpha=1.0, out=None, beta=0.0,
            precision=0):
        a = A.T if transA else A
        b = B.T if transB else B
        return alpha * ((a.conj() if conjA else a) @ (b.conj() if conjB else b))

    def bdot(X, Y):
        return (X.reshape(X.shape[0], -1) * Y.reshape(Y.shape[0], -1)).sum(-1)
    monkeypatch.setattr(spatial, "zmm", zmm)
    monkeypatch.setattr(spatial, "bdot", bdot)


def _problem(n, no, seed):
    rng = np.random.default_rng(seed)
    L = 3 * n
    A = rng.standard_normal((L, n, n)) + 1j * rng.standard_normal((L, n, n))
    A = (A + np.conj(A.transpose(0, 2, 1))) / (2 * np.sqrt(n * L))
    eri = np.einsum("Lpq,Lrs->pqrs", A, A)                     # chemist, Hermitian factors
    eps = np.sort(np.concatenate([rng.uniform(-1.5, -0.3, no), rng.uniform(0.2, 3.0, n - no)]))
    F = np.diag(eps).astype(complex) + 0.02 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return F, eri, eps


def test_spatial_residual_matches_oracle(torch_gemm):
    n, no = 9, 3
    F, eri, _ = _problem(n, no, 1)
    rng = np.random.default_rng(2)
    nv = n - no
    t1 = 0.1 * (rng.standard_normal((no, nv)) + 1j * rng.standard_normal((no, nv)))
    t2 = 0.1 * (rng.standard_normal((no, no, nv, nv)) + 1j * rng.standard_normal((no, no, nv, nv)))
    t2 = t2 + t2.transpose(1, 0, 3, 2)                         # closed-shell symmetry t_ijab = t_jiba
    E = 0.2 - 0.05j
    eng = spatial.SpatialCISD(torch.as_tensor(F), torch.as_tensor(eri), no)
    r1, r2 = eng.residual(torch.as_tensor(t1), torch.as_tensor(t2), E)
    q1, q2 = port.cisd_spatial_residual(F, eri, t1, t2, E, no)
    np.testing.assert_allclose(r1.numpy(), q1, atol=1e-13, rtol=0)
    np.testing.assert_allclose(r2.numpy(), q2, atol=1e-13, rtol=0)
    eng2 = spatial.SpatialCISD(torch.as_tensor(F), torch.as_tensor(eri), no, singles=False)
    _, r2c = eng2.residual(None, torch.as_tensor(t2), E)
    np.testing.assert_allclose(r2c.numpy(), port.cid_spatial_residual(F, eri, t2, E, no), atol=1e-13, rtol=0)


def test_spatial_solve_matches_spin_orbital_oracle(torch_gemm):
    n, no = 8, 3
    F, eri, eps = _problem(n, no, 3)
    F = np.diag(eps).astype(complex)
    P = dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-12)
    blk = port.blocks_from_chemist(port.compute_ERI_SO(eri), 2 * no)
    Er, t1r, t2r = port.solve_cisd_so(port.compute_F_SO(F), blk, eps[:no], eps[no:], P)
    for singles in (True, False):
        eng = spatial.SpatialCISD(torch.as_tensor(F), torch.as_tensor(eri), no, singles=singles)
        eng.set_denominators(eps[:no], eps[no:])
        E, t1, t2 = eng.solve(P)
        if singles:
            assert abs(E - Er) < 1e-11
            np.testing.assert_allclose(t2.numpy(), t2r[0::2, 1::2, 0::2, 1::2], atol=1e-9, rtol=0)
            np.testing.assert_allclose(t1.numpy(), t1r[0::2, 0::2], atol=1e-9, rtol=0)
        else:
            Ec, _ = port.solve_cisd_so(port.compute_F_SO(F), blk, eps[:no], eps[no:], P, singles=False)
            assert abs(E - Ec) < 1e-11
