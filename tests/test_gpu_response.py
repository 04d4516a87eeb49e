"""First-order CISD_SO / CID_SO amplitude response (apyib/analytic_aats.py:757-875 in spin
orbitals): t^x and E^x from solve_response against central differences of full GPU solves
at F + lambda dF, ERI(B + lambda dB), combined by Richardson extrapolation (steps 1e-4 and
5e-5), on seeded synthetic problems with a complex Hermitian Fock perturbation and a
perturbation of the Hermitian factors."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import synthetic  # noqa: E402
from apyib_gb300.cisd import CISDPlan, solve  # noqa: E402
from apyib_gb300.response import solve_response  # noqa: E402

P = dict(max_iterations=200, DIIS=True, e_convergence=1e-13, d_convergence=1e-12)


def chem(B1, B2):
    return np.einsum("Lpq,Lrs->pqrs", B1, B2)


def make_plan(o, v, F, eri, eps_so, singles, mixed=False):
    plan = CISDPlan(o, v, singles=singles, mixed=mixed)
    plan.set_fock(torch.as_tensor(F), eps_so)
    plan.blocks_from_so(torch.as_tensor(eri))
    return plan


@pytest.mark.parametrize("singles", [True, False], ids=["cisd", "cid"])
def test_response_matches_central_differences(singles):
    o, v = 4, 10
    prob = synthetic.so_factors(o, v, seed=31)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    n = o + v
    rng = np.random.default_rng(32)
    F0 = prob.fock_so()
    X = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.01
    mask = np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2 == 0
    F0 = F0 + (X + X.conj().T) * mask                      # non-Brillouin: every Fock term counts
    Y = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.3
    dF = (Y + Y.conj().T) * mask
    Z = rng.standard_normal(prob.B.shape) + 1j * rng.standard_normal(prob.B.shape)
    dB = (Z + np.conj(Z.transpose(0, 2, 1))) / 2 * (0.3 / np.sqrt(n * prob.B.shape[0]))
    B = prob.B
    plan = make_plan(o, v, F0, chem(B, B), eps_so, singles)
    E, t = solve(plan, P)
    plan_x = make_plan(o, v, dF, chem(dB, B) + chem(B, dB), eps_so, singles)
    dE, dt = solve_response(plan, plan_x, t, E, P)

    def at(lam):
        Bl = B + lam * dB
        p = make_plan(o, v, F0 + lam * dF, chem(Bl, Bl), eps_so, singles)
        return solve(p, P)

    def fd(h):
        (Ep, tp), (Em, tm) = at(h), at(-h)
        return (Ep - Em) / (2 * h), (tp - tm) / (2 * h)
    e1, t1 = fd(1e-4)
    e2, t2 = fd(5e-5)
    e_fd, t_fd = (4 * e2 - e1) / 3, (4 * t2 - t1) / 3
    assert abs(dE - e_fd) <= 1e-7 * abs(e_fd) + 1e-10, (dE, e_fd)
    scale = t_fd.abs().max().item()
    assert (dt - t_fd).abs().max().item() <= 1e-7 * scale + 1e-10


def test_response_ozaki_matches_fp64():
    """The FP64-accurate tensor-core residual gives the same response as the FP64 one."""
    o, v = 20, 80
    prob = synthetic.so_factors(o, v, seed=33)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    n = o + v
    rng = np.random.default_rng(34)
    Y = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.1
    mask = np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2 == 0
    dF = (Y + Y.conj().T) * mask
    plan = CISDPlan(o, v, mixed=True)
    plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    plan_x = CISDPlan(o, v, mixed=True)
    plan_x.set_fock(torch.as_tensor(dF), eps_so)
    plan_x.blocks_from_factors(torch.as_tensor(prob.B * 0.0))
    E, t = solve(plan, P)
    dE64, dt64 = solve_response(plan, plan_x, t, E, P, precision="fp64")
    dEoz, dtoz = solve_response(plan, plan_x, t, E, P, precision="ozaki")
    assert abs(dE64 - dEoz) < 1e-10 * max(1.0, abs(dE64))
    assert (dt64 - dtoz).abs().max().item() < 1e-9 * max(1.0, dt64.abs().max().item())


@pytest.mark.parametrize("diis", [True, False])
def test_lockstep_responses_match_one_at_a_time(diis):
    """solve_responses (several perturbations in lockstep, converging at different
    iterations) gives each response exactly what solve_response gives it alone."""
    from apyib_gb300.response import solve_responses
    o, v = 4, 8
    prob = synthetic.so_factors(o, v, seed=41)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    n = o + v
    mask = np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2 == 0
    rng = np.random.default_rng(42)
    B = prob.B
    plan = make_plan(o, v, prob.fock_so(), chem(B, B), eps_so, True)
    params = dict(P, DIIS=diis, max_iterations=80)
    E, t = solve(plan, params)
    pxs = []
    for k, s in enumerate((0.05, 0.3, 1.0)):
        Y = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * s
        Z = rng.standard_normal(B.shape) + 1j * rng.standard_normal(B.shape)
        dB = (Z + np.conj(Z.transpose(0, 2, 1))) / 2 * (s / np.sqrt(n * B.shape[0]))
        pxs.append(make_plan(o, v, (Y + Y.conj().T) * mask, chem(dB, B) + chem(B, dB), eps_so, True))
    hist_all = [[] for _ in pxs]
    together = solve_responses(plan, pxs, t, E, params, histories=hist_all)
    for k, px in enumerate(pxs):
        hist = []
        dE, dt = solve_response(plan, px, t, E, params, history=hist)
        assert len(hist) == len(hist_all[k])
        assert abs(together[k][0] - dE) <= 1e-14 * max(1.0, abs(dE))
        assert torch.abs(together[k][1] - dt).max().item() <= 1e-14 * max(1.0, torch.abs(dt).max().item())
