"""One CISD_SO iteration at o/v = 40/160 (nso = 200, naux = 800) against the
unmodified reference: tests/golden/make_golden_c3.py ran apyib/ci_wfn.py:263-337
with a lazy ERI_SO stand-in on the same seeded inputs, with a non-diagonal complex
Fock matrix.  Compared: t1 after the iteration in full, t2 at 4096 seeded probes,
three seeded random projections of t2, |t2|^2 and the energy.  The GPU path runs
the FP64 residual through the C ABI (blocks from the factors in FP64), and the
Ozaki (tensor-core, FP64-accurate) residual on the same plan."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib, synthetic  # noqa: E402
from apyib_gb300.cisd import CISDPlan  # noqa: E402
from tests.golden.c3_case import (FIXTURE, NPROBE, O, SEED, V, digest, perturbed_fock,  # noqa: E402
                                  probe_indices, projection_weights)
from tests.gpu_util import load_gold  # noqa: E402


@pytest.fixture(scope="module")
def case():
    g = load_gold(FIXTURE)
    prob = synthetic.so_factors(O, V, seed=SEED)
    Fp = perturbed_fock(prob, O, V, SEED)
    assert digest(prob.B, prob.eps_o, prob.eps_v, Fp) == str(g["input_sha"]), "input generator drifted"
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    plan = CISDPlan(O, V, mixed=True)
    plan.set_fock(torch.as_tensor(Fp), eps_so)
    plan.blocks_from_factors(torch.as_tensor(prob.B))
    return g, plan


@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_OZAKI], ids=["fp64", "ozaki"])
def test_c3_iteration_matches_reference(case, prec):
    g, plan = case
    t = plan.guess()
    E0, _, _ = plan.combine([t], [1.0], t, t)
    r = plan.residual(t, E0, prec)
    plan.check_status()
    tn = plan.update(t, r)
    E1, _, _ = plan.combine([tn], [1.0], tn, tn)
    t1, t2 = plan.unpack(tn)
    t1 = t1.cpu().numpy()
    np.testing.assert_allclose(t1, g["t1_iter1"], atol=1e-12, rtol=0)
    idx = probe_indices(O, V, NPROBE, SEED + 1)
    np.testing.assert_array_equal(idx, g["probe_idx"])
    it = torch.as_tensor(idx, device=t2.device)
    probes = t2[it[0], it[1], it[2], it[3]].cpu().numpy()
    np.testing.assert_allclose(probes, g["t2_probes"], atol=1e-12, rtol=0)
    for k in range(3):
        w = torch.as_tensor(projection_weights(O, V, SEED + 2 + k), device=t2.device)
        proj = complex(torch.sum(w * t2).item())
        assert abs(proj - complex(g["t2_proj"][k])) < 1e-10 * max(1.0, abs(complex(g["t2_proj"][k])))
    assert abs(torch.sum(t2.abs() ** 2).item() - float(g["t2_norm2"])) < 1e-10 * float(g["t2_norm2"])
    assert abs(E1 - complex(g["E_iter1"])) < 1e-11


def test_c3_tf32x3_residual_tracks_fp64(case):
    """The 3xTF32 residual (every singles GEMM with o = 40 as its narrow, transposed-store
    side) against the FP64 residual on the same amplitudes: FP32-level agreement."""
    _, plan = case
    t = plan.guess()
    E0, _, _ = plan.combine([t], [1.0], t, t)
    r64 = plan.residual(t, E0, _lib.PREC_FP64)
    r32 = plan.residual(t, E0, _lib.PREC_TF32X3)
    plan.check_status()
    n1 = O * V
    for part in (slice(0, n1), slice(n1, None)):
        ref = r64[part]
        err = (r32[part] - ref).abs().max().item() / ref.abs().max().item()
        assert err < 2e-5, err
