"""GPU CISD_SO / CID_SO / MP2_SO parity against the reference-pinned oracle
and the golden fixtures.  FP64 mode: energies to 1e-10 Eh, amplitudes to
1e-9 max-abs.  Mixed mode: |dE| <= 1e-9 Eh against the FP64 result."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib, synthetic  # noqa: E402
from apyib_gb300.cisd import CISDPlan  # noqa: E402
from apyib_gb300.ci_wfn import solve_so_system  # noqa: E402
from oracle import port  # noqa: E402
from tests.gpu_util import load_gold, so_golden_files  # noqa: E402

P = dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-13)


def prob_of(g):
    return synthetic.so_factors(int(g["o"]), int(g["v"]), seed=int(g["seed"]), real=bool(g["real"]))


@pytest.mark.parametrize("path", so_golden_files(with_inputs=True), ids=os.path.basename)
@pytest.mark.parametrize("source", ["factors", "so", "mo_like"])
def test_single_residual_matches_reference(path, source):
    g = load_gold(os.path.basename(path))
    prob = prob_of(g)
    o, v = prob.o, prob.v
    plan = CISDPlan(o, v)
    F = g["F_pert"]
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(F), eps_so)
    eri = np.einsum("Lpq,Lrs->pqrs", prob.B, prob.B)
    if source == "factors":
        plan.blocks_from_factors(torch.as_tensor(prob.B))
    else:
        plan.blocks_from_so(torch.as_tensor(eri))
    t = plan.guess()
    E0, _, _ = plan.combine([t], [1.0], t, t)
    r = plan.residual(t, E0)
    t1n = plan.update(t, r)
    t1, t2 = plan.unpack(t1n)
    np.testing.assert_allclose(t1.cpu().numpy(), g["t1_iter1"], atol=1e-13, rtol=0)
    np.testing.assert_allclose(t2.cpu().numpy(), g["t2_iter1"], atol=1e-13, rtol=0)


@pytest.mark.parametrize("path", so_golden_files(), ids=os.path.basename)
def test_solves_match_reference(path):
    g = load_gold(os.path.basename(path))
    prob = prob_of(g)
    F = prob.fock_so()
    E, t1, t2 = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B)
    assert abs(E - g["E_cisd"]) < 1e-10
    np.testing.assert_allclose(t1.cpu().numpy(), g["t1_cisd"], atol=1e-9, rtol=0)
    if "t2_cisd" in g:
        np.testing.assert_allclose(t2.cpu().numpy(), g["t2_cisd"], atol=1e-9, rtol=0)
    E, _, t2 = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B, singles=False)
    assert abs(E - g["E_cid"]) < 1e-10
    plan = CISDPlan(prob.o, prob.v, mp2_only=True)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(F), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    E, t = plan.mp2()
    assert abs(E - g["E_mp2"]) < 1e-12
    if "t2_mp2" in g:
        _, t2 = plan.unpack(t)
        np.testing.assert_allclose(t2.cpu().numpy(), g["t2_mp2"], atol=1e-12)


@pytest.mark.parametrize("o,v,seed", [(8, 30, 31), (12, 44, 32)])
def test_solve_matches_oracle_larger(o, v, seed):
    prob = synthetic.so_factors(o, v, seed=seed)
    blk = port.blocks_from_factors(prob.B, o)
    F = prob.fock_so()
    Er, t1r, t2r = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P)
    E, t1, t2 = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B)
    assert abs(E - Er) < 1e-10
    assert np.abs(t2.cpu().numpy() - t2r).max() < 1e-9
    assert np.abs(t1.cpu().numpy() - t1r).max() < 1e-9


def test_nondiagonal_fock_solve_matches_oracle():
    prob = synthetic.so_factors(6, 14, seed=41)
    rng = np.random.default_rng(0)
    F = prob.fock_so()
    n = prob.nso
    pert = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.003
    pert = pert + pert.conj().T
    mask = (np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2) == 0
    F = F + pert * mask
    blk = port.blocks_from_factors(prob.B, prob.o)
    Er, t1r, t2r = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P)
    E, t1, t2 = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B)
    assert abs(E - Er) < 1e-10
    assert np.abs(t2.cpu().numpy() - t2r).max() < 1e-9


@pytest.mark.parametrize("base,singles,offdiag", [("ozaki", True, False), ("df64", True, False),
                                                   ("fp64", True, False), ("ozaki", False, False),
                                                   ("ozaki", True, True)])
def test_mixed_precision_reaches_fp64_energy(base, singles, offdiag):
    """Mixed solves (3xTF32 iterations, defect correction around one FP64-accurate residual)
    reach the FP64 solve for every base precision, for CID, and with a non-diagonal complex
    Fock matrix (every Fock term of the residual active)."""
    from apyib_gb300.cisd import solve
    prob = synthetic.so_factors(20, 80, seed=7)
    F = prob.fock_so()
    if offdiag:
        n = F.shape[0]
        rng = np.random.default_rng(8)
        X = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.01
        mask = np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2 == 0
        F = F + (X + X.conj().T) * mask
    p = dict(P, e_convergence=1e-12, d_convergence=1e-10)
    res = solve_so_system(F, prob.eps_o, prob.eps_v, p, B=prob.B, singles=singles)
    E64, t2_64 = res[0], res[-1]
    plan = CISDPlan(prob.o, prob.v, singles=singles, mixed=True)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(F), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    hist = []
    Em, t = solve(plan, p, precision="mixed", history=hist, base_precision=base)
    _, t2_m = plan.unpack(t)
    assert abs(Em - E64) < 1e-9, (Em, E64, hist)
    assert np.abs(t2_m.cpu().numpy() - t2_64.cpu().numpy()).max() < 1e-8


def test_df64_residual_matches_fp64_residual():
    prob = synthetic.so_factors(12, 44, seed=9)
    plan = CISDPlan(prob.o, prob.v)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    t = plan.guess()
    r64 = plan.residual(t, 0.1 - 0.01j, _lib.PREC_FP64)
    rdf = plan.residual(t, 0.1 - 0.01j, _lib.PREC_DF64)
    err = (rdf - r64).abs().max().item() / r64.abs().max().item()
    assert err < 1e-11, err


@pytest.mark.parametrize("o,v,offdiag", [(6, 30, True), (20, 80, True), (64, 96, False), (70, 100, True)])
def test_tf32x3_residual_tracks_fp64(o, v, offdiag):
    """3xTF32 residual against the FP64 residual on the same amplitudes (every term,
    singles included): o <= 64 takes the 64-wide tile and the transposed stores for the
    singles GEMMs, o = 70 the 256-wide tile over the same transposed orientation."""
    prob = synthetic.so_factors(o, v, seed=o + v)
    F = prob.fock_so()
    if offdiag:
        n = F.shape[0]
        rng = np.random.default_rng(o)
        X = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.01
        mask = np.add.outer(np.arange(n) % 2, np.arange(n) % 2) % 2 == 0
        F = F + (X + X.conj().T) * mask
    plan = CISDPlan(o, v, mixed=True)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(F), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    t = plan.guess()
    torch.manual_seed(o)
    t = t + 0.01 * torch.randn_like(t)          # singles non-zero
    E0, _, _ = plan.combine([t], [1.0], t, t)
    r64 = plan.residual(t, E0, _lib.PREC_FP64)
    r32 = plan.residual(t, E0, _lib.PREC_TF32X3)
    plan.check_status()
    n1 = o * v
    for part in (slice(0, n1), slice(n1, None)):
        ref = r64[part]
        err = (r32[part] - ref).abs().max().item() / ref.abs().max().item()
        assert err < 2e-5, err


def test_plan_gemm_timing_is_per_plan():
    """The GEMM timing log belongs to the plan that switched it on: a 3xTF32 residual
    records its tcgen05 launches there and nowhere else, and collecting clears it."""
    import ctypes
    o, v = 20, 80
    prob = synthetic.so_factors(o, v, seed=3)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plans = []
    for _ in range(2):
        plan = CISDPlan(o, v, mixed=True)
        plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
        plan.blocks_from_factors(torch.as_tensor(prob.B))
        plans.append(plan)
    timed, other = plans
    _lib.call("agb_cisd_plan_gemm_timing", timed._h, 1)
    t = timed.guess()
    E0, _, _ = timed.combine([t], [1.0], t, t)
    timed.residual(t, E0, _lib.PREC_TF32X3)
    other.residual(t, E0, _lib.PREC_TF32X3)
    _lib.call("agb_cisd_plan_gemm_timing", timed._h, 0)

    def collect(plan):
        n, ms, fl = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        _lib.call("agb_cisd_plan_gemm_timing_collect", plan._h, 0.0, ctypes.byref(n), ctypes.byref(ms),
                  ctypes.byref(fl))
        return n.value, ms.value, fl.value

    n, ms, fl = collect(timed)
    assert n > 0 and ms > 0.0 and fl >= 8.0 * (o * v) ** 3       # at least the ring product
    assert collect(timed) == (0, 0.0, 0.0)                       # cleared
    assert collect(other) == (0, 0.0, 0.0)                       # never switched on
    for plan in plans:
        plan.check_status()
