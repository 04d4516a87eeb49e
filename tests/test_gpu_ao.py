"""GPU SCF (J/K), AO->MO transform and the full SCF -> CISD_SO / MP2_SO
pipeline against fixtures generated by the reference itself."""
import glob
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402
from apyib_gb300.ci_wfn import ci_wfn  # noqa: E402
from apyib_gb300.hamiltonian import Hamiltonian  # noqa: E402
from apyib_gb300.hf_wfn import hf_wfn  # noqa: E402
from apyib_gb300.mp2_wfn import mp2_wfn  # noqa: E402
from apyib_gb300 import utils  # noqa: E402
from tests.gpu_util import GOLD  # noqa: E402

FILES = sorted(glob.glob(os.path.join(GOLD, "ao_*.npz")))


def params(method, fc):
    return dict(method=method, e_convergence=1e-13, d_convergence=1e-13, DIIS=True, freeze_core=fc,
                max_iterations=100, F_el=[0, 0, 0], F_mag=[0, 0, 0])


def make(g):
    H = Hamiltonian.from_arrays(g["T"], g["V"], g["S"], g["ERI"], float(g["E_nuc"]), nelec=2 * int(g["ndocc"]),
                                nfzc=int(g["nfzc"]))
    return H


@pytest.mark.parametrize("path", FILES, ids=os.path.basename)
def test_scf_matches_reference(path):
    g = dict(np.load(path))
    fc = int(g["nfzc"]) > 0
    wfn = hf_wfn(make(g))
    E, C = wfn.solve_SCF(params("RHF", fc))
    assert abs(E - g["E_scf"]) < 1e-10
    np.testing.assert_allclose(wfn.eps, g["eps"], atol=1e-9)


@pytest.mark.parametrize("path", FILES, ids=os.path.basename)
def test_transforms_and_correlated_energies(path):
    g = dict(np.load(path))
    fc = int(g["nfzc"]) > 0
    wfn = hf_wfn(make(g))
    wfn.solve_SCF(params("RHF", fc))
    # continue from the reference's orbitals so phases match the fixtures
    wfn.C = g["C"]
    wfn.eps = g["eps"]
    wfn.E_SCF = g["E_scf"]
    p = params("CISD_SO", fc)
    C_list, I_list = utils.get_slices(p, wfn)
    F_MO, E_fc = utils.compute_F_MO(p, wfn, C_list)
    np.testing.assert_allclose(F_MO, g["F_MO"], atol=1e-11)
    assert abs(E_fc - g["E_fc"]) < 1e-11
    ERI_MO = utils.compute_ERI_MO(p, wfn, C_list)
    np.testing.assert_allclose(ERI_MO, g["ERI_MO"], atol=1e-12)
    E, t1, t2 = ci_wfn(p, wfn).solve_CISD_SO()
    assert abs(E - g["E_cisd"]) < 1e-10
    np.testing.assert_allclose(t2, g["t2_cisd"], atol=1e-9)
    E, t2 = ci_wfn(params("CID_SO", fc), wfn).solve_CID_SO()
    assert abs(E - g["E_cid"]) < 1e-10
    E, t2 = mp2_wfn(params("MP2_SO", fc), wfn).solve_MP2_SO()
    assert abs(E - g["E_mp2"]) < 1e-10
    np.testing.assert_allclose(t2, g["t2_mp2"], atol=1e-9)
    E, t2 = mp2_wfn(params("MP2", fc), wfn).solve_MP2()
    assert abs(E - g["E_mp2_spatial"]) < 1e-10
    np.testing.assert_allclose(t2, g["t2_mp2_spatial"], atol=1e-9)
    E, t1, t2 = ci_wfn(params("CISD", fc), wfn).solve_CISD()
    assert abs(E - g["E_cisd_spatial"]) < 1e-10
    np.testing.assert_allclose(t1, g["t1_cisd_spatial"], atol=1e-9)
    np.testing.assert_allclose(t2, g["t2_cisd_spatial"], atol=1e-9)
    E, t2 = ci_wfn(params("CID", fc), wfn).solve_CID()
    assert abs(E - g["E_cid_spatial"]) < 1e-10
    np.testing.assert_allclose(t2, g["t2_cid_spatial"], atol=1e-9)


@pytest.mark.parametrize("path", FILES, ids=os.path.basename)
def test_mixed_precision_through_ci_wfn(path):
    """parameters['precision'] = 'mixed' through the drop-in class: tensor-core
    iterations plus defect correction reach the reference energy to 1e-9 Eh."""
    g = dict(np.load(path))
    fc = int(g["nfzc"]) > 0
    wfn = hf_wfn(make(g))
    wfn.solve_SCF(params("RHF", fc))
    wfn.C, wfn.eps, wfn.E_SCF = g["C"], g["eps"], g["E_scf"]
    p = dict(params("CISD_SO", fc), precision="mixed", e_convergence=1e-12, d_convergence=1e-10)
    E, t1, t2 = ci_wfn(p, wfn).solve_CISD_SO()
    assert abs(E - g["E_cisd"]) < 1e-9
    np.testing.assert_allclose(t2, g["t2_cisd"], atol=1e-8)
    E, t2 = ci_wfn(dict(p, method="CID_SO"), wfn).solve_CID_SO()
    assert abs(E - g["E_cid"]) < 1e-9


@pytest.mark.parametrize("prec,tol", [(_lib.PREC_DF64, 1e-12), (_lib.PREC_OZAKI, 1e-11), (_lib.PREC_TF32X3, 2e-6)])
def test_transform_precision_modes(prec, tol):
    """The double-float, Ozaki and 3xTF32 transforms (the first quarter step reads the
    real AO integrals directly) against the reference's ERI_MO fixture."""
    g = dict(np.load(FILES[0]))
    fc = int(g["nfzc"]) > 0
    wfn = hf_wfn(make(g))
    wfn.C = g["C"]
    wfn.eps = g["eps"]
    p = params("CISD_SO", fc)
    C_list, _ = utils.get_slices(p, wfn)
    ERI_MO = utils.compute_ERI_MO(p, wfn, C_list, precision=prec)
    scale = np.abs(g["ERI_MO"]).max()
    np.testing.assert_allclose(ERI_MO, g["ERI_MO"], atol=tol * scale)


@pytest.mark.parametrize("n", [40, 70])
def test_transform_tf32x3_matches_fp64_multi_tile(n):
    """The 3xTF32 transform (the GEMMs convert the FP64 intermediate in their own
    converter warps; nmo = 40 takes the 64-wide tile, 70 the 160-wide one, thousands of
    128-row tiles) against the FP64 transform of the same seeded AO integrals.  Bound:
    each quarter step carries ~2^-21 of sum |a||b| (~sqrt(n) times its result for a
    unitary C), four steps chained: 1e-5 of the largest element."""
    import ctypes

    from apyib_gb300.device import ptr, stream_ptr, workspace
    g = torch.Generator(device="cpu").manual_seed(n)
    A = torch.randn(2 * n, n, n, generator=g, dtype=torch.float64)
    A = ((A + A.transpose(1, 2)) / (2 * (2 * n * n) ** 0.5)).cuda()
    eri = torch.einsum("Lmn,Lls->mnls", A, A).contiguous()
    Cm = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.complex128))[0].cuda().contiguous()
    out = {}
    for prec in (_lib.PREC_FP64, _lib.PREC_TF32X3):
        o = torch.empty(n, n, n, n, dtype=torch.complex128, device="cuda")
        nb = _lib.load().agb_ao2mo_scratch_bytes(n, n, prec)
        buf, sp, _ = workspace(nb)
        _lib.call("agb_ao2mo", ptr(eri), n, ptr(Cm), n, ptr(o), ctypes.c_void_p(sp), ctypes.c_size_t(nb), prec,
                  stream_ptr())
        torch.cuda.synchronize()
        out[prec] = o
        del buf
    scale = out[_lib.PREC_FP64].abs().max().item()
    err = (out[_lib.PREC_TF32X3] - out[_lib.PREC_FP64]).abs().max().item() / scale
    assert err < 1e-5, err


def test_transform_tf32x3_256_wide_tile():
    """nmo = 168 (> 160) puts every quarter step of the 3xTF32 transform on the converter
    GEMM's 256-wide tile (Re and Im accumulators filling TMEM's 512 columns, two stages);
    nbf = 20 keeps K and the intermediates small (the output is 168^4 complex, 12.7 GB).
    Against the Ozaki transform (FP64-accurate; the FP64 GEMM's grid does not reach
    168^3 rows), bound as in the multi-tile test: 1e-5 of the largest element."""
    import ctypes

    from apyib_gb300.device import ptr, stream_ptr, workspace
    nbf, nmo = 20, 168
    g = torch.Generator(device="cpu").manual_seed(7)
    A = torch.randn(2 * nbf, nbf, nbf, generator=g, dtype=torch.float64)
    A = ((A + A.transpose(1, 2)) / (2 * (2 * nbf * nbf) ** 0.5)).cuda()
    eri = torch.einsum("Lmn,Lls->mnls", A, A).contiguous()
    Cm = (torch.randn(nbf, nmo, generator=g, dtype=torch.complex128) / nbf ** 0.5).cuda().contiguous()
    out = {}
    for prec in (_lib.PREC_OZAKI, _lib.PREC_TF32X3):
        o = torch.empty(nmo, nmo, nmo, nmo, dtype=torch.complex128, device="cuda")
        nb = _lib.load().agb_ao2mo_scratch_bytes(nbf, nmo, prec)
        buf, sp, _ = workspace(nb)
        _lib.call("agb_ao2mo", ptr(eri), nbf, ptr(Cm), nmo, ptr(o), ctypes.c_void_p(sp), ctypes.c_size_t(nb), prec,
                  stream_ptr())
        torch.cuda.synchronize()
        out[prec] = o
        del buf
    scale = out[_lib.PREC_OZAKI].abs().max().item()
    err = (out[_lib.PREC_TF32X3] - out[_lib.PREC_OZAKI]).abs().max().item() / scale
    assert err < 1e-5, err
