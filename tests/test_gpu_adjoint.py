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
    D, G = densities(plan, t, vo_coupling=True)     # the reference's exact CISD densities
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
    # every spin-allowed Fock element, including the ov / vo blocks (the backward uses
    # the solver-consistent D_vo; see apyib_gb300.adjoint)
    # (scaled so the O(h^2) truncation of the central difference stays below 1e-6 relative at h = 1e-4)
    dF = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * mask * 0.05
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


def test_core_hamiltonian_backward_matches_central_differences():
    """dE/dh at fixed orbitals against central differences of full GPU pipelines
    (F_MO from h, ERI_MO, SO blocks, CISD_SO solve) along a magnetic-field-like
    Hermitian direction dh = i * L / 2 (L real antisymmetric)."""
    import os
    import types
    from apyib_gb300.adjoint import cisd_energy_core
    from apyib_gb300.hamiltonian import Hamiltonian
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "ao_8_3_0_f.npz")))
    H = Hamiltonian.from_arrays(g["T"], g["V"], g["S"], g["ERI"], float(g["E_nuc"]), nelec=2 * int(g["ndocc"]))
    wfn = types.SimpleNamespace(H=H, C=g["C"], eps=g["eps"], ndocc=int(g["ndocc"]), nbf=int(g["nbf"]))
    params = dict(method="CISD_SO", e_convergence=1e-13, d_convergence=1e-12, DIIS=True, freeze_core=False,
                  max_iterations=100)
    h0 = g["T"] + g["V"]
    rng = np.random.default_rng(3)
    Lz = rng.standard_normal(h0.shape)
    dh = 1j * (Lz - Lz.T) / 2 * 0.5
    ht = torch.tensor(h0, device="cuda", requires_grad=True)
    E = cisd_energy_core(ht, wfn, params)
    E.real.backward()
    pred = np.real(np.sum(np.conj(ht.grad.cpu().numpy()) * dh))
    h = 1e-4

    def E_at(s):
        return cisd_energy_core(torch.tensor(h0 + s * dh, device="cuda"), wfn, params).real.item()
    fd = (E_at(h) - E_at(-h)) / (2 * h)
    assert abs(fd - pred) <= 1e-6 * abs(pred) + 1e-10, (fd, pred)


@pytest.mark.parametrize("name", ["ao_8_3_0_f.npz", "ao_9_4_1_f.npz"])
def test_mo_coefficient_gradient_matches_central_differences(name):
    """dE/dC and dE/dC* (Wirtinger) of the CISD_SO energy against central differences of
    full GPU pipelines (F_MO with J/K from the occupied / frozen-core densities of C,
    the AO->MO transform with C, SO blocks, CISD_SO solve) along random complex changes
    of the virtual and of the occupied columns (their contributions cancel in part when
    mixed, which would blur a relative check); the frozen-core case exercises the
    density term of the frozen orbitals."""
    import os
    import types
    from apyib_gb300.adjoint import mo_coefficient_gradient
    from apyib_gb300.hamiltonian import Hamiltonian
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name)))
    nfzc = int(g["nfzc"])
    H = Hamiltonian.from_arrays(g["T"], g["V"], g["S"], g["ERI"], float(g["E_nuc"]), nelec=2 * int(g["ndocc"]),
                                nfzc=nfzc)
    params = dict(method="CISD_SO", e_convergence=1e-13, d_convergence=1e-12, DIIS=True, freeze_core=nfzc > 0,
                  max_iterations=100)
    h0 = g["T"] + g["V"]

    def wfn_at(C):
        return types.SimpleNamespace(H=H, C=C, eps=g["eps"], ndocc=int(g["ndocc"]), nbf=int(g["nbf"]))
    E0, dC, dCc = mo_coefficient_gradient(h0, wfn_at(g["C"]), params)
    dC, dCc = dC.cpu().numpy(), dCc.cpu().numpy()
    rng = np.random.default_rng(5)
    d = (rng.standard_normal(g["C"].shape) + 1j * rng.standard_normal(g["C"].shape)) * 0.1

    def E_at(x):
        return mo_coefficient_gradient(h0, wfn_at(g["C"] + x), params)[0]
    # virtual columns, then occupied + frozen-core columns (whose J/K density term enters);
    # central differences at h = 1e-4 and 5e-5 combined by Richardson extrapolation
    ndocc = int(g["ndocc"])
    for cols in (slice(ndocc, None), slice(0, ndocc)):
        dd = np.zeros_like(d)
        dd[:, cols] = d[:, cols]
        pred = np.sum(dC * dd) + np.sum(dCc * np.conj(dd))
        f1 = (E_at(1e-4 * dd) - E_at(-1e-4 * dd)) / 2e-4
        f2 = (E_at(5e-5 * dd) - E_at(-5e-5 * dd)) / 1e-4
        fd = (4 * f2 - f1) / 3
        assert abs(fd - pred) <= 1e-6 * abs(pred) + 1e-10, (cols, fd, pred)
