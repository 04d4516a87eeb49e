"""Adjoint (density) gradients of the CISD_SO energy on the GPU.

Checks: (1) the GPU densities equal the oracle's (the reference's own
adjoint formulas, apyib/ci_wfn.py:382-411); (2) E = sum F D + sum <pq|rs> G;
(3) the autograd backward agrees with central finite differences of full
solves (steps 1e-4 and 1e-5) along random directions in F and in the
Hermitian ERI factors, to <= 1e-6 relative."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import synthetic  # noqa: E402
from apyib_gb300.adjoint import cisd_energy, densities, energy_from_densities, gamma_full  # noqa: E402
from apyib_gb300.ci_wfn import solve_so_system  # noqa: E402
from oracle import port  # noqa: E402

P = dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-12)


def chem(B):
    return np.einsum("Lpq,Lrs->pqrs", B, B)


@pytest.mark.parametrize("o,v,seed", [(4, 8, 21), (6, 10, 22)])
def test_densities_match_oracle_and_energy(o, v, seed):
    prob = synthetic.so_factors(o, v, seed=seed)
    F = prob.fock_so()
    E, t, plan = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B, return_plan=True)
    D, G = densities(plan, t)
    t1, t2 = plan.unpack(t)
    Dr, Gr = port.cisd_so_densities(t1.cpu().numpy(), t2.cpu().numpy(), o, o + v)
    np.testing.assert_allclose(D.cpu().numpy(), Dr, atol=1e-12)
    Gf = gamma_full(G, o, v).cpu().numpy()
    np.testing.assert_allclose(Gf, Gr, atol=1e-12)
    Ead = energy_from_densities(torch.as_tensor(F).cuda(), torch.as_tensor(chem(prob.B)).cuda(),
                                D, torch.as_tensor(Gf).cuda())
    assert abs(complex(Ead) - E) < 1e-10


@pytest.mark.parametrize("h", [1e-4, 1e-5])
def test_backward_matches_central_differences(h):
    o, v = 4, 10
    prob = synthetic.so_factors(o, v, seed=23)
    rng = np.random.default_rng(5)
    n = o + v
    F = prob.fock_so()
    mask = (np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2) == 0
    # occupied-occupied and virtual-virtual blocks only: the reference's doubles
    # equations (apyib/ci_wfn.py:319-334) omit the F_ov t1 coupling, so its energy is
    # stationary (Hellmann-Feynman) only for F_ov = 0, as with canonical orbitals.
    occ = np.arange(n) < o
    mask = mask & (np.equal.outer(occ, occ))
    dF = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask
    dF = dF + dF.conj().T
    X = rng.standard_normal(prob.B.shape) + 1j * rng.standard_normal(prob.B.shape)
    dB = (X + np.conj(X.transpose(0, 2, 1))) / 2 * 1e-2
    Ft = torch.tensor(F, device="cuda", requires_grad=True)
    Et = torch.tensor(chem(prob.B), device="cuda", requires_grad=True)
    E = cisd_energy(Ft, Et, prob.eps_o, prob.eps_v, P)
    E.real.backward()
    gF, gE = Ft.grad.cpu().numpy(), Et.grad.cpu().numpy()
    dERI = np.einsum("Lpq,Lrs->pqrs", dB, prob.B) + np.einsum("Lpq,Lrs->pqrs", prob.B, dB)
    # PyTorch convention: dL = Re(sum conj(grad) * dz)
    pred = np.real(np.sum(np.conj(gF) * dF) + np.sum(np.conj(gE) * dERI))

    def E_at(s):
        B = prob.B + s * dB
        Es, _, _ = solve_so_system(F + s * dF, prob.eps_o, prob.eps_v, P, ERI_SO=chem(B))
        return Es.real
    fd = (E_at(h) - E_at(-h)) / (2 * h)
    assert abs(fd - pred) <= 1e-6 * max(abs(pred), 1e-8) + 1e-9, (fd, pred)
