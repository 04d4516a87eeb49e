"""Pin the NumPy oracle (oracle/port.py) to fixtures produced by the
unmodified reference (tests/golden/make_golden.py).  CPU only."""
import glob
import os

import numpy as np
import pytest

from apyib_gb300 import synthetic
from oracle import port

GOLD = os.path.join(os.path.dirname(__file__), "golden")
P = dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-13)


def so_cases():
    return sorted(glob.glob(os.path.join(GOLD, "so_*.npz")))


def load_so(path):
    g = dict(np.load(path))
    o, v, seed, real = int(g["o"]), int(g["v"]), int(g["seed"]), bool(g["real"])
    prob = synthetic.so_factors(o, v, seed=seed, real=real)
    if "B" in g:
        np.testing.assert_array_equal(prob.B, g["B"])     # generator drift check
    return g, prob


@pytest.mark.parametrize("path", so_cases(), ids=os.path.basename)
def test_so_solves_match_reference(path):
    g, prob = load_so(path)
    o = prob.o
    blk = port.blocks_from_factors(prob.B, o)
    F = prob.fock_so()
    E, t1, t2 = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P)
    assert abs(E - g["E_cisd"]) < 1e-12
    np.testing.assert_allclose(t1, g["t1_cisd"], atol=1e-12, rtol=0)
    if "t2_cisd" in g:
        np.testing.assert_allclose(t2, g["t2_cisd"], atol=1e-12, rtol=0)
    E, t2 = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P, singles=False)
    assert abs(E - g["E_cid"]) < 1e-12
    E, t2 = port.solve_mp2_so(blk, prob.eps_o, prob.eps_v)
    assert abs(E - g["E_mp2"]) < 1e-13


@pytest.mark.parametrize("path", [p for p in so_cases() if "F_pert" in dict(np.load(p))], ids=os.path.basename)
def test_single_residual_matches_reference(path):
    g, prob = load_so(path)
    o = prob.o
    blk = port.blocks_from_factors(prob.B, o)
    F = g["F_pert"]
    D_ia, D_ijab = port.so_denominators(prob.eps_o, prob.eps_v)
    Oo, Vv = slice(0, o), slice(o, None)
    t1 = F.T[Oo, Vv] / D_ia
    t2 = blk["vvoo"].transpose(2, 3, 0, 1) / D_ijab
    E0 = np.einsum("ia,ia->", t1, F[Oo, Vv]) + 0.25 * np.einsum("ijab,ijab->", t2, blk["oovv"])
    r1, r2 = port.cisd_so_residual(F, blk, t1, t2, E0, o)
    np.testing.assert_allclose(t1 + r1 / D_ia, g["t1_iter1"], atol=1e-13, rtol=0)
    np.testing.assert_allclose(t2 + r2 / D_ijab, g["t2_iter1"], atol=1e-13, rtol=0)


def test_chemist_block_builder_matches_factor_builder():
    prob = synthetic.so_factors(4, 6, seed=9)
    eri = np.einsum("Lpq,Lrs->pqrs", prob.B, prob.B)
    a = port.blocks_from_chemist(eri, 4)
    b = port.blocks_from_factors(prob.B, 4)
    for k in port.BLOCKS:
        np.testing.assert_allclose(a[k], b[k], atol=1e-14)


def test_diis_matches_reference():
    g = np.load(os.path.join(GOLD, "diis.npz"))
    e_iter = t_iter = None
    for it in range(1, len(g["r"]) + 1):
        r, t = g["r"][it - 1], g["t"][it - 1]
        if it == 1:
            t_iter = t.reshape(-1, 1)
            e_iter = r.reshape(-1, 1)
        tv, e_iter, t_iter = port.solve_general_DIIS(r, t, e_iter, t_iter, it)
        np.testing.assert_allclose(tv, g["tv"][it - 1], atol=1e-12)
    assert e_iter.shape[1] == 8      # truncation to 7, then append


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "ao_*.npz"))), ids=os.path.basename)
def test_ao_pipeline_matches_reference(path):
    g = dict(np.load(path))
    nbf, ndocc, nfzc = int(g["nbf"]), int(g["ndocc"]), int(g["nfzc"])
    E, C, eps = port.solve_scf(g["T"], g["V"], g["S"], g["ERI"], float(g["E_nuc"]), ndocc,
                               dict(max_iterations=100, DIIS=True, e_convergence=1e-13, d_convergence=1e-13))
    assert abs(E - g["E_scf"]) < 1e-11
    np.testing.assert_allclose(eps, g["eps"], atol=1e-10)
    C = g["C"]                         # continue from the reference's orbitals (phase-fixed)
    F_MO, E_fc = port.compute_F_MO(g["T"] + g["V"], g["ERI"], C, nfzc, ndocc, nbf, freeze_core=nfzc > 0)
    np.testing.assert_allclose(F_MO, g["F_MO"], atol=1e-11)
    assert abs(E_fc - g["E_fc"]) < 1e-11
    ERI_MO = port.compute_ERI_MO(g["ERI"], C[:, nfzc:])
    np.testing.assert_allclose(ERI_MO, g["ERI_MO"], atol=1e-12)
    F_SO = port.compute_F_SO(F_MO)
    eri_so = port.compute_ERI_SO(ERI_MO)
    o = 2 * (ndocc - nfzc)
    blk = port.blocks_from_chemist(eri_so, o)
    eps_o, eps_v = g["eps"][nfzc:ndocc], g["eps"][ndocc:]
    E, t1, t2 = port.solve_cisd_so(F_SO, blk, eps_o, eps_v, P)
    assert abs(E - g["E_cisd"]) < 1e-11
    np.testing.assert_allclose(t2, g["t2_cisd"], atol=1e-10)
    E, t2 = port.solve_mp2_so(blk, eps_o, eps_v)
    assert abs(E - g["E_mp2"]) < 1e-11


def test_adjoint_densities_reproduce_energy():
    """The density form of apyib/ci_wfn.py:382-411 reproduces the converged
    CISD_SO correlation energy (the reference's own stated check)."""
    prob = synthetic.so_factors(4, 8, seed=21)
    o, n = prob.o, prob.nso
    B = prob.B
    eri = np.einsum("Lpq,Lrs->pqrs", B, B)
    blk = port.blocks_from_chemist(eri, o)
    F = prob.fock_so()
    E, t1, t2 = port.solve_cisd_so(F, blk, prob.eps_o, prob.eps_v, P)
    D, G = port.cisd_so_densities(t1, t2, o, n)
    dirac = eri.transpose(0, 2, 1, 3)
    # Normal-ordered: subtract the occupied reference part of F.
    E_adj = np.einsum("pq,pq->", F, D) + np.einsum("pqrs,pqrs->", dirac, G)
    assert abs(E_adj - E) < 1e-10


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "ao_*.npz"))), ids=os.path.basename)
def test_spatial_mp2_matches_reference(path):
    g = dict(np.load(path))
    nfzc, ndocc = int(g["nfzc"]), int(g["ndocc"])
    E, t2 = port.solve_mp2_spatial(g["ERI_MO"], g["eps"][nfzc:ndocc], g["eps"][ndocc:])
    assert abs(E - g["E_mp2_spatial"]) < 1e-12
    np.testing.assert_allclose(t2, g["t2_mp2_spatial"], atol=1e-13)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "ao_*.npz"))), ids=os.path.basename)
def test_spatial_cisd_is_the_alpha_beta_block_of_the_so_solution(path):
    """The reference's closed-shell spatial CISD / CID (apyib/ci_wfn.py:51-167,
    420-574) give the same energies as its spin-orbital solvers, with
    t1 = t1_SO[alpha, alpha] and t2 = t2_SO[alpha, beta, alpha, beta]."""
    g = dict(np.load(path))
    assert abs(g["E_cisd_spatial"] - g["E_cisd"]) < 1e-12
    assert abs(g["E_cid_spatial"] - g["E_cid"]) < 1e-12
    np.testing.assert_allclose(g["t2_cisd"][0::2, 1::2, 0::2, 1::2], g["t2_cisd_spatial"], atol=1e-13)
    np.testing.assert_allclose(g["t1_cisd"][0::2, 0::2], g["t1_cisd_spatial"], atol=1e-13)


@pytest.mark.parametrize("a0,a1", [(0, 2), (3, 7), (9, 10)])
def test_virtual_row_sample_equals_rows_of_the_full_residual(a0, a1):
    """The CPU baseline times rows a0 <= a < a1 of the residual (every reference einsum
    restricted to those output rows); they must be exactly those rows of the full one,
    on a complex non-diagonal Fock matrix and random amplitudes."""
    prob = synthetic.so_factors(6, 10, seed=3)
    o, n = prob.o, prob.nso
    rng = np.random.default_rng(4)
    F = prob.fock_so() + 0.05 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    t1 = 0.1 * (rng.standard_normal((o, prob.v)) + 1j * rng.standard_normal((o, prob.v)))
    t2 = 0.1 * (rng.standard_normal((o, o, prob.v, prob.v)) + 1j * rng.standard_normal((o, o, prob.v, prob.v)))
    t2 = t2 - t2.transpose(1, 0, 2, 3)
    t2 = t2 - t2.transpose(0, 1, 3, 2)
    E = 0.3 - 0.1j
    r1, r2 = port.cisd_so_residual(F, port.blocks_from_factors(prob.B, o), t1, t2, E, o)
    blk = port.vslab_blocks_from_factors(prob.B, o, a0, a1)
    for lay in (None, port.vslab_layouts(blk, t2)):
        s1, s2 = port.cisd_so_residual_vslab(F, blk, t1, t2, E, o, a0, a1, lay=lay)
        np.testing.assert_allclose(s1, r1[:, a0:a1], atol=1e-13, rtol=0)
        np.testing.assert_allclose(s2, r2[:, :, a0:a1, :], atol=1e-13, rtol=0)
