"""Edge cases and size-independent properties of the GPU CISD path."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib, synthetic  # noqa: E402
from apyib_gb300.cisd import CISDPlan, solve  # noqa: E402
from apyib_gb300.ci_wfn import solve_so_system  # noqa: E402
from oracle import port  # noqa: E402

P = dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-13)


@pytest.mark.parametrize("o,v", [(2, 2), (2, 6), (8, 2), (2, 34), (14, 4)])
def test_extreme_shapes_match_oracle(o, v):
    prob = synthetic.so_factors(o, v, seed=o * 100 + v)
    blk = port.blocks_from_factors(prob.B, o)
    F = prob.fock_so()
    Er, t1r, t2r = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P)
    E, t1, t2 = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B)
    assert abs(E - Er) < 1e-10
    assert np.abs(t2.cpu().numpy() - t2r).max() < 1e-9
    Er2, _ = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P, singles=False)
    E2, _, _ = solve_so_system(F, prob.eps_o, prob.eps_v, P, B=prob.B, singles=False)
    assert abs(E2 - Er2) < 1e-10


def test_pack_unpack_round_trip_and_antisymmetry():
    o, v = 6, 10
    plan = CISDPlan(o, v)
    rng = np.random.default_rng(1)
    t2 = rng.standard_normal((o, o, v, v)) + 1j * rng.standard_normal((o, o, v, v))
    t2 = t2 - t2.transpose(1, 0, 2, 3)
    t2 = t2 - t2.transpose(0, 1, 3, 2)
    t1 = rng.standard_normal((o, v)) + 1j * rng.standard_normal((o, v))
    t = plan.pack(torch.as_tensor(t1), torch.as_tensor(t2))
    u1, u2 = plan.unpack(t)
    np.testing.assert_array_equal(u1.cpu().numpy(), t1)
    np.testing.assert_array_equal(u2.cpu().numpy(), t2)


def test_workspace_errors_are_reported():
    h = ctypes.c_void_p()
    _lib.call("agb_cisd_plan_create", 4, 6, 0, ctypes.byref(h))
    buf = torch.empty(1024, dtype=torch.uint8, device="cuda")
    with pytest.raises(_lib.AGBError) as e:
        _lib.call("agb_cisd_plan_set_workspace", h, ctypes.c_void_p(buf.data_ptr()), ctypes.c_size_t(1024))
    assert e.value.status == _lib.AGB_ERR_WORKSPACE
    _lib.load().agb_cisd_plan_destroy(h)


def test_not_converged_prints_and_returns(capsys):
    prob = synthetic.so_factors(4, 8, seed=3)
    p = dict(P, max_iterations=2)
    E, t1, t2 = solve_so_system(prob.fock_so(), prob.eps_o, prob.eps_v, p, B=prob.B)
    assert "Not converged." in capsys.readouterr().out
    assert np.isfinite(E)


def test_full_size_properties_40_160():
    """At o/v = 40/160 (no FP64 oracle in seconds): the mixed solution satisfies the
    FP64 residual equations, the energy of the Hermitian problem is real, and the
    double-float residual agrees with the FP64 one."""
    prob = synthetic.so_factors(40, 160, seed=0)
    plan = CISDPlan(40, 160, mixed=True)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    p = dict(P, e_convergence=1e-11, d_convergence=1e-9)
    E, t = solve(plan, p, precision="mixed")
    r64 = plan.residual(t, E, _lib.PREC_FP64)
    corr = plan.update(torch.zeros_like(t), r64)
    assert corr.abs().max().item() < 1e-9
    assert abs(E.imag) < 1e-12
    rdf = plan.residual(t, E, _lib.PREC_DF64)
    assert (rdf - r64).abs().max().item() < 1e-11 * max(1.0, r64.abs().max().item()) + 1e-13


def test_checkpoint_resume_reaches_same_energy(tmp_path):
    prob = synthetic.so_factors(6, 14, seed=8)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])

    def plan_():
        p = CISDPlan(prob.o, prob.v)
        p.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
        p.blocks_from_factors(torch.as_tensor(prob.B))
        return p
    E_full, _ = solve(plan_(), P)
    ck = str(tmp_path / "ck.npz")
    E_part, _ = solve(plan_(), dict(P, max_iterations=2), checkpoint=ck, checkpoint_every=2)
    E_res, _ = solve(plan_(), P, checkpoint=ck, resume=True)
    assert abs(E_res - E_full) < 1e-11
    assert abs(E_part - E_full) > 1e-11         # the truncated run had not converged
    assert int(np.load(ck)["iteration"]) > 2    # the resumed run kept checkpointing
