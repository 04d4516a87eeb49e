"""Adjoint of the MP2_SO energy (apyib_gb300.adjoint: the Hylleraas Lagrangian of
apyib/mp2_wfn.py:64-87's energy, its densities and the MP2Energy autograd.Function).

Checks: (1) at a diagonal Fock matrix the energy is the oracle's MP2_SO energy
(oracle/port.py, pinned to the reference) and E = sum F D + sum <pq|rs> Gamma;
(2) the non-canonical amplitudes solve their equations; (3) the backward agrees with
central finite differences of the energy (steps 1e-4 and 1e-5) along random Hermitian
directions in every spin-allowed Fock block and in the ERI factors, to 1e-6 relative."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import synthetic  # noqa: E402
from apyib_gb300.adjoint import (energy_from_densities, gamma_full, mp2_densities, mp2_energy,  # noqa: E402
                                 mp2_lagrangian_solve, mp2_so_blocks, _mp2_fock_offdiag, _mp2_denominators)
from oracle import port  # noqa: E402


def chem(B):
    return np.einsum("Lpq,Lrs->pqrs", B, B)


@pytest.mark.parametrize("o,v,seed", [(4, 8, 31), (6, 10, 32)])
def test_mp2_energy_and_densities_match_oracle(o, v, seed):
    prob = synthetic.so_factors(o, v, seed=seed)
    F = torch.as_tensor(prob.fock_so()).cuda()
    eri = torch.as_tensor(chem(prob.B)).cuda()
    W, V = mp2_so_blocks(eri, o)
    E, t, lam = mp2_lagrangian_solve(F, W, V, o)
    Er, t2r = port.solve_mp2_so(port.blocks_from_factors(prob.B, o), prob.eps_o, prob.eps_v)
    assert abs(E - Er) < 1e-12
    np.testing.assert_allclose(t.cpu().numpy(), t2r, atol=1e-13, rtol=0)
    np.testing.assert_allclose(lam.cpu().numpy(), np.conj(t2r), atol=1e-13, rtol=0)   # Hermitian integrals
    D, G = mp2_densities(t, lam)
    Ead = energy_from_densities(F, eri, D, gamma_full(G, o, v))
    assert abs(complex(Ead) - E) < 1e-12


def test_noncanonical_amplitudes_solve_their_equations():
    o, v = 4, 8
    prob = synthetic.so_factors(o, v, seed=33)
    rng = np.random.default_rng(1)
    n = o + v
    mask = (np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2) == 0
    dF = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask * 0.02
    F = torch.as_tensor(prob.fock_so() + dF + dF.conj().T).cuda()
    W, V = mp2_so_blocks(torch.as_tensor(chem(prob.B)).cuda(), o)
    E, t, lam = mp2_lagrangian_solve(F, W, V, o)
    Foo, Fvv = F[:o, :o], F[o:, o:]
    D = _mp2_denominators(Foo, Fvv)
    r = V - D * t + _mp2_fock_offdiag(t, Foo, Fvv)
    rl = W - D * lam + _mp2_fock_offdiag(lam, Foo, Fvv, transpose=True)
    assert r.abs().max().item() < 1e-12 and rl.abs().max().item() < 1e-12
    # the Lagrangian densities still reproduce the energy away from the canonical point
    Dn, G = mp2_densities(t, lam)
    Ead = energy_from_densities(F, torch.as_tensor(chem(prob.B)).cuda(), Dn, gamma_full(G, o, v))
    assert abs(complex(Ead) - E) < 1e-12


@pytest.mark.parametrize("h", [1e-4, 1e-5])
def test_mp2_backward_matches_central_differences(h):
    o, v = 4, 10
    prob = synthetic.so_factors(o, v, seed=34)
    rng = np.random.default_rng(6)
    n = o + v
    F = prob.fock_so()
    mask = (np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2) == 0
    dF = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask * 0.05
    dF = dF + dF.conj().T
    X = rng.standard_normal(prob.B.shape) + 1j * rng.standard_normal(prob.B.shape)
    dB = (X + np.conj(X.transpose(0, 2, 1))) / 2 * 1e-2
    Ft = torch.tensor(F, device="cuda", requires_grad=True)
    Et = torch.tensor(chem(prob.B), device="cuda", requires_grad=True)
    E = mp2_energy(Ft, Et, o)
    E.real.backward()
    gF, gE = Ft.grad.cpu().numpy(), Et.grad.cpu().numpy()
    dERI = np.einsum("Lpq,Lrs->pqrs", dB, prob.B) + np.einsum("Lpq,Lrs->pqrs", prob.B, dB)
    pred = np.real(np.sum(np.conj(gF) * dF) + np.sum(np.conj(gE) * dERI))

    def E_at(s):
        B = prob.B + s * dB
        return complex(mp2_energy(torch.as_tensor(F + s * dF).cuda(), torch.as_tensor(chem(B)).cuda(), o)).real
    fd = (E_at(h) - E_at(-h)) / (2 * h)
    assert abs(fd - pred) <= 1e-6 * max(abs(pred), 1e-8) + 1e-9, (fd, pred)
