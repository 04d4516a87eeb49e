"""The MP2_SO Lagrangian algebra of apyib_gb300.adjoint (amplitude and multiplier
equations, densities, the MP2Energy backward) is tensor algebra around the library's
complex GEMM.  With that GEMM pointed at torch on the CPU it runs here: the energy must
equal the oracle's MP2_SO energy (pinned to apyib/mp2_wfn.py:64-87), the densities
must reproduce it, and the backward must agree with central differences of the energy
in Fock and ERI directions (the GPU twin of this test, test_gpu_mp2_adjoint.py, runs
the same checks through the CUDA library)."""
import numpy as np
import pytest
import torch

from apyib_gb300 import adjoint as adj
from apyib_gb300 import synthetic
from oracle import port


@pytest.fixture
def torch_gemm(monkeypatch):
    def zmm(A, B, transA=False, conjA=False, transB=False, conjB=False, alpha=1.0, out=None, beta=0.0,
            precision=0):
        a = A.T if transA else A
        b = B.T if transB else B
        return alpha * ((a.conj() if conjA else a) @ (b.conj() if conjB else b))
    monkeypatch.setattr(adj, "zmm", zmm)


def chem(B):
    return np.einsum("Lpq,Lrs->pqrs", B, B)


def test_mp2_lagrangian_on_cpu(torch_gemm):
    o, v = 4, 10
    prob = synthetic.so_factors(o, v, seed=34)
    F = torch.as_tensor(prob.fock_so())
    eri = torch.as_tensor(chem(prob.B))
    W, V = adj.mp2_so_blocks(eri, o)
    E, t, lam = adj.mp2_lagrangian_solve(F, W, V, o)
    Er, t2r = port.solve_mp2_so(port.blocks_from_factors(prob.B, o), prob.eps_o, prob.eps_v)
    assert abs(E - Er) < 1e-13
    np.testing.assert_allclose(t.numpy(), t2r, atol=1e-14, rtol=0)
    D, G = adj.mp2_densities(t, lam)
    assert abs(complex(adj.energy_from_densities(F, eri, D, adj.gamma_full(G, o, v))) - E) < 1e-13
    rng = np.random.default_rng(6)
    n = o + v
    mask = (np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2) == 0
    dF = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask * 0.05
    dF = dF + dF.conj().T
    X = rng.standard_normal(prob.B.shape) + 1j * rng.standard_normal(prob.B.shape)
    dB = (X + np.conj(X.transpose(0, 2, 1))) / 2 * 1e-2
    Ft = torch.tensor(prob.fock_so(), requires_grad=True)
    Et = torch.tensor(chem(prob.B), requires_grad=True)
    adj.MP2Energy.apply(Ft, Et, o).real.backward()
    dERI = np.einsum("Lpq,Lrs->pqrs", dB, prob.B) + np.einsum("Lpq,Lrs->pqrs", prob.B, dB)
    pred = np.real(np.sum(np.conj(Ft.grad.numpy()) * dF) + np.sum(np.conj(Et.grad.numpy()) * dERI))

    def E_at(s):
        Fs = torch.as_tensor(prob.fock_so() + s * dF)
        return complex(adj.MP2Energy.apply(Fs, torch.as_tensor(chem(prob.B + s * dB)), o)).real
    h = 1e-5
    fd = (E_at(h) - E_at(-h)) / (2 * h)
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)
