"""CPU restatement (NumPy) of apyib's correlated-wavefunction hot path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: the parity tests, the
``smoke()`` self-check and the CPU-baseline leg of ``bench.py`` may call it,
as the checker; the product path (``apyib_gb300``) never imports it.

Every function restates one reference function and cites it.  Reference paths
are relative to the apyib project root.  The restatement is pinned against
the reference itself: ``tests/golden/make_golden.py`` runs the unmodified
reference modules (with a stub psi4) on seeded inputs and
``tests/test_oracle_golden.py`` checks this module against those fixtures.

Conventions (as in the reference):
  * spin orbitals interleave alpha (even index) and beta (odd index)
    (apyib/utils.py:294-311, 332-363);
  * chemist ERIs (pq|rs); Dirac <pq|rs> = (pr|qs) (apyib/ci_wfn.py:284);
  * <pq||rs> = <pq|rs> - <pq|sr>;
  * complex energies and norms are NOT conjugated (apyib/ci_wfn.py:293,355,361-365).
"""
from __future__ import annotations

import numpy as np

# ----------------------------------------------------------------------------
# Spin-orbital expansion and slices
# ----------------------------------------------------------------------------


def get_slices(method: str, nbf: int, ndocc: int, nfzc: int = 0):
    """apyib/utils.py:184-213 (wfn attributes passed explicitly)."""
    C_list = [slice(0, nfzc), slice(nfzc, ndocc), slice(ndocc, nbf), slice(nfzc, nbf)]
    if method in ("RHF", "MP2", "CID", "CISD"):
        I_list = [slice(0, nfzc), slice(0, ndocc - nfzc), slice(ndocc - nfzc, nbf - nfzc), slice(0, nbf - nfzc)]
    elif method in ("MP2_SO", "CID_SO", "CISD_SO"):
        I_list = [slice(0, 2 * nfzc), slice(0, 2 * ndocc - 2 * nfzc),
                  slice(2 * ndocc - 2 * nfzc, 2 * nbf - 2 * nfzc), slice(0, 2 * nbf - 2 * nfzc)]
    else:
        raise ValueError(method)
    return C_list, I_list


def compute_F_SO(F_MO):
    """apyib/utils.py:283-313: F_SO[p,q] = F_MO[p//2,q//2] if spin(p)==spin(q) else 0."""
    n = F_MO.shape[0]
    F_SO = np.zeros((2 * n, 2 * n), dtype=F_MO.dtype)
    F_SO[0::2, 0::2] = F_MO
    F_SO[1::2, 1::2] = F_MO
    return F_SO


def compute_ERI_SO(ERI_MO):
    """apyib/utils.py:317-365: chemist ERI_SO[p,q,r,s] = ERI_MO[p//2,q//2,r//2,s//2]
    when spin(p)==spin(q) and spin(r)==spin(s), else 0."""
    n0, n1, n2, n3 = ERI_MO.shape
    out = np.zeros((2 * n0, 2 * n1, 2 * n2, 2 * n3), dtype=ERI_MO.dtype)
    for sp in (0, 1):
        for sr in (0, 1):
            out[sp::2, sp::2, sr::2, sr::2] = ERI_MO
    return out


# ----------------------------------------------------------------------------
# Antisymmetrised Dirac blocks
# ----------------------------------------------------------------------------

BLOCKS = ("oovv", "vvoo", "ovvo", "vovv", "ooov", "ovoo", "vvvo", "oooo", "vvvv")


def dirac_as_block(eri_chem, sl):
    """<pq||rs> for index ranges sl=(P,Q,R,S) from a chemist tensor:
    <pq|rs> = (pr|qs) (apyib/ci_wfn.py:284), minus the r<->s exchange."""
    P, Q, R, S = sl
    direct = eri_chem[P, R, Q, S].transpose(0, 2, 1, 3)
    exch = eri_chem[P, S, Q, R].transpose(0, 2, 3, 1)
    return direct - exch


def blocks_from_chemist(eri_chem, o: int):
    """All antisymmetrised blocks the CISD_SO residual reads, from a full
    spin-orbital chemist tensor with the first ``o`` indices occupied."""
    n = eri_chem.shape[0]
    O = slice(0, o)
    V = slice(o, n)
    m = {"o": O, "v": V}
    return {name: dirac_as_block(eri_chem, tuple(m[c] for c in name)) for name in BLOCKS}


def blocks_from_factors(B, o: int, names=BLOCKS):
    """Antisymmetrised blocks from Hermitian factors B[L,p,q]:
    (pq|rs) = sum_L B[L,p,q] * conj(B[L,s,r]) = sum_L B[L,p,q] * B[L,r,s]."""
    n = B.shape[1]
    O = slice(0, o)
    V = slice(o, n)
    m = {"o": O, "v": V}
    out = {}
    for name in names:
        P, Q, R, S = (m[c] for c in name)
        # <pq|rs> = (pr|qs) = sum_L B[L,p,r] B[L,q,s]
        direct = np.einsum("Lpr,Lqs->pqrs", B[:, P, R], B[:, Q, S], optimize=True)
        exch = np.einsum("Lps,Lqr->pqrs", B[:, P, S], B[:, Q, R], optimize=True)
        out[name] = direct - exch
    return out


# ----------------------------------------------------------------------------
# DIIS
# ----------------------------------------------------------------------------


def solve_general_DIIS(res_vec, t_vec, e_iter, t_iter, iteration, max_DIIS=7):
    """apyib/utils.py:104-140.  e_iter/t_iter are (length, nvec) matrices.
    Truncation to max_DIIS happens before the append (:109-112), so up to
    max_DIIS+1 vectors enter B; iteration 1 does not append (:117)."""
    while e_iter.shape[1] > max_DIIS:
        e_iter = e_iter[:, 1:]
        t_iter = t_iter[:, 1:]
    if iteration != 1:
        e_iter = np.hstack((e_iter, res_vec.reshape(-1, 1)))
        t_iter = np.hstack((t_iter, t_vec.reshape(-1, 1)))
    Bm = e_iter.conj().T @ e_iter
    nb = Bm.shape[0]
    B = np.zeros((nb + 1, nb + 1), dtype=Bm.dtype)
    B[:nb, :nb] = Bm
    B[-1, :] = -1
    B[:, -1] = -1
    B[-1, -1] = 0
    A = np.zeros(nb + 1)
    A[-1] = -1
    c = np.linalg.solve(B, A)
    return t_iter @ c[:-1], e_iter, t_iter


def diis_coefficients(Bm):
    """The bordered DIIS solve of apyib/utils.py:121-135 for a given Gram
    matrix Bm = e^H e; returns the nvec extrapolation weights."""
    nb = Bm.shape[0]
    B = np.zeros((nb + 1, nb + 1), dtype=np.result_type(Bm, np.complex128))
    B[:nb, :nb] = Bm
    B[-1, :] = -1
    B[:, -1] = -1
    B[-1, -1] = 0
    A = np.zeros(nb + 1)
    A[-1] = -1
    return np.linalg.solve(B, A)[:-1]


# ----------------------------------------------------------------------------
# Residuals
# ----------------------------------------------------------------------------


def cisd_so_residual(F, blk, t1, t2, E, o: int, singles: bool = True):
    """T1/T2 residuals of apyib/ci_wfn.py:309-334 (singles=True) or
    :210-220 (CID_SO, singles=False).  F is the full F_SO; blk holds the
    antisymmetrised Dirac blocks."""
    O = slice(0, o)
    V = slice(o, F.shape[0])
    Foo, Fvv, Fov = F[O, O], F[V, V], F[O, V]
    ein = lambda s, *a: np.einsum(s, *a, optimize=True)
    r1 = None
    if singles:
        r1 = F.T[O, V].copy()
        r1 -= ein("ji,ja->ia", Foo, t1)
        r1 += ein("ab,ib->ia", Fvv, t1)
        r1 += ein("jabi,jb->ia", blk["ovvo"], t1)
        r1 += ein("jb,ijab->ia", Fov, t2)
        r1 += 0.5 * ein("ajcb,ijcb->ia", blk["vovv"], t2)
        r1 -= 0.5 * ein("kjib,kjab->ia", blk["ooov"], t2)
        r1 -= E * t1
    r2 = blk["vvoo"].transpose(2, 3, 0, 1).copy()
    if singles:
        r2 -= ein("kbij,ka->ijab", blk["ovoo"], t1)
        r2 -= ein("akij,kb->ijab", -blk["ovoo"].transpose(1, 0, 2, 3), t1)
        r2 += ein("abcj,ic->ijab", blk["vvvo"], t1)
        r2 += ein("abic,jc->ijab", -blk["vvvo"].transpose(0, 1, 3, 2), t1)
    r2 += ein("bc,ijac->ijab", Fvv, t2)
    r2 += ein("ac,ijcb->ijab", Fvv, t2)
    r2 -= ein("kj,ikab->ijab", Foo, t2)
    r2 -= ein("ki,kjab->ijab", Foo, t2)
    r2 += 0.5 * ein("klij,klab->ijab", blk["oooo"], t2)
    r2 += 0.5 * ein("abcd,ijcd->ijab", blk["vvvv"], t2)
    W = blk["ovvo"]
    r2 += ein("kbcj,ikac->ijab", W, t2)
    r2 += ein("kbci,kjac->ijab", W, t2)
    r2 += ein("kacj,ikcb->ijab", W, t2)
    r2 += ein("kaci,kjcb->ijab", W, t2)
    r2 -= E * t2
    return r1, r2


VSLAB_SPEC = {"ovvo": "ovvo", "ooov": "ooov", "ovoo": "ovoo", "oooo": "oooo",
              "vvvv": "avvv", "vovv": "aovv", "vvvo": "avvo", "vvoo": "avoo"}


def vslab_blocks_from_factors(B, o: int, a0: int, a1: int, names=tuple(VSLAB_SPEC)):
    """The antisymmetrised blocks ``cisd_so_residual_vslab`` reads for the residual rows
    a0 <= a < a1 (virtual index): ovvo, ooov, ovoo and oooo in full, and vvvv, vovv,
    vvvo, vvoo with their first (virtual) index restricted to [a0, a1).  Same formula
    as ``blocks_from_factors``; ``names`` selects blocks."""
    n = B.shape[1]
    m = {"o": slice(0, o), "v": slice(o, n), "a": slice(o + a0, o + a1)}
    out = {}
    for name in names:
        ranges = VSLAB_SPEC[name]
        P, Q, R, S = (m[c] for c in ranges)
        direct = np.einsum("Lpr,Lqs->pqrs", B[:, P, R], B[:, Q, S], optimize=True)
        exch = np.einsum("Lps,Lqr->pqrs", B[:, P, S], B[:, Q, R], optimize=True)
        out[name] = direct - exch
    return out


def vslab_layouts(blk, t2):
    """Full-size operands of ``cisd_so_residual_vslab`` laid out once in the order its
    contractions read them (the ring integrals as [b, j, k, c]; t2 as [c, i, j, b],
    [k, c, i, b] and [k, c, j, b]), so that a timed row sample copies nothing of full
    size: einsum would otherwise re-lay these out on every call, a cost the full
    residual pays once per term, not once per sampled row block."""
    W = blk["ovvo"]
    return {"W_bjkc": np.ascontiguousarray(W.transpose(1, 3, 0, 2)),
            "t2_cijb": np.ascontiguousarray(t2.transpose(2, 0, 1, 3)),
            "t2_kcib": np.ascontiguousarray(t2.transpose(1, 2, 0, 3)),
            "t2_kcjb": np.ascontiguousarray(t2.transpose(0, 2, 1, 3))}


def cisd_so_residual_vslab(F, blk, t1, t2, E, o: int, a0: int, a1: int, lay=None):
    """Rows a0 <= a < a1 of ``cisd_so_residual`` (apyib/ci_wfn.py:309-334): r1[:, a0:a1]
    and r2[:, :, a0:a1, :], every einsum of the reference restricted to those output
    rows with its full contraction lengths, so the work is (a1 - a0) / v of each term.
    ``blk`` comes from ``vslab_blocks_from_factors`` (or has the same slices); ``lay``
    (from ``vslab_layouts``) gives the full-size operands pre-laid-out."""
    O = slice(0, o)
    V = slice(o, F.shape[0])
    A = slice(a0, a1)
    Foo, Fvv, Fov = F[O, O], F[V, V], F[O, V]
    ein = lambda s, *a: np.einsum(s, *a, optimize=True)
    t1a, t2a = t1[:, A], t2[:, :, A, :]
    W = blk["ovvo"]
    r1 = F.T[O, V][:, A].copy()
    r1 -= ein("ji,ja->ia", Foo, t1a)
    r1 += ein("ab,ib->ia", Fvv[A], t1)
    r1 += ein("jabi,jb->ia", W[:, A], t1)
    r1 += ein("jb,ijab->ia", Fov, t2a)
    r1 += 0.5 * ein("ajcb,ijcb->ia", blk["vovv"], t2)
    r1 -= 0.5 * ein("kjib,kjab->ia", blk["ooov"], t2a)
    r1 -= E * t1a
    r2 = blk["vvoo"].transpose(2, 3, 0, 1).copy()
    r2 -= ein("kbij,ka->ijab", blk["ovoo"], t1a)
    r2 -= ein("akij,kb->ijab", -blk["ovoo"][:, A].transpose(1, 0, 2, 3), t1)
    r2 += ein("abcj,ic->ijab", blk["vvvo"], t1)
    r2 += ein("abic,jc->ijab", -blk["vvvo"].transpose(0, 1, 3, 2), t1)
    r2 += ein("bc,ijac->ijab", Fvv, t2a)
    if lay is None:
        r2 += ein("ac,ijcb->ijab", Fvv[A], t2)
    else:
        r2 += ein("ac,cijb->ijab", Fvv[A], lay["t2_cijb"])
    r2 -= ein("kj,ikab->ijab", Foo, t2a)
    r2 -= ein("ki,kjab->ijab", Foo, t2a)
    r2 += 0.5 * ein("klij,klab->ijab", blk["oooo"], t2a)
    r2 += 0.5 * ein("abcd,ijcd->ijab", blk["vvvv"], t2)
    if lay is None:
        r2 += ein("kbcj,ikac->ijab", W, t2a)
        r2 += ein("kbci,kjac->ijab", W, t2a)
        r2 += ein("kacj,ikcb->ijab", W[:, A], t2)
        r2 += ein("kaci,kjcb->ijab", W[:, A], t2)
    else:
        r2 += ein("bjkc,ikac->ijab", lay["W_bjkc"], t2a)
        r2 += ein("bikc,kjac->ijab", lay["W_bjkc"], t2a)
        r2 += ein("kacj,kcib->ijab", W[:, A], lay["t2_kcib"])
        r2 += ein("kaci,kcjb->ijab", W[:, A], lay["t2_kcjb"])
    r2 -= E * t2a
    return r1, r2


def cisd_spatial_residual(F, ERI_MO, t1, t2, E, no: int, singles: bool = True):
    """Closed-shell T1/T2 residuals of apyib/ci_wfn.py:458-490 (CISD; t1 ignored and
    r1 None for CID, :84-111) for the active-space F_MO and chemist ERI_MO."""
    O, V = slice(0, no), slice(no, F.shape[0])
    g = ERI_MO.swapaxes(1, 2)
    gx = g.swapaxes(2, 3)
    ein = lambda s, *a: np.einsum(s, *a, optimize=True)
    r1 = None
    if singles:
        r1 = F.swapaxes(0, 1)[O, V].copy()
        r1 -= ein("ji,ja->ia", F[O, O], t1)
        r1 += ein("ab,ib->ia", F[V, V], t1)
        r1 += ein("jabi,jb->ia", 2.0 * g[O, V, V, O] - gx[O, V, V, O], t1)
        r1 += ein("jb,ijab->ia", F[O, V], 2.0 * t2 - t2.swapaxes(2, 3))
        r1 += ein("ajbc,ijbc->ia", 2.0 * g[V, O, V, V] - gx[V, O, V, V], t2)
        r1 -= ein("kjib,kjab->ia", 2.0 * g[O, O, O, V] - gx[O, O, O, V], t2)
        r1 -= E * t1
    r2 = g.swapaxes(0, 2).swapaxes(1, 3)[O, O, V, V].copy()
    if singles:
        r2 += ein("abcj,ic->ijab", g[V, V, V, O], t1)
        r2 += ein("abic,jc->ijab", g[V, V, O, V], t1)
        r2 -= ein("kbij,ka->ijab", g[O, V, O, O], t1)
        r2 -= ein("akij,kb->ijab", g[V, O, O, O], t1)
    r2 += ein("ac,ijcb->ijab", F[V, V], t2)
    r2 += ein("bc,ijac->ijab", F[V, V], t2)
    r2 -= ein("ki,kjab->ijab", F[O, O], t2)
    r2 -= ein("kj,ikab->ijab", F[O, O], t2)
    r2 += ein("klij,klab->ijab", g[O, O, O, O], t2)
    r2 += ein("abcd,ijcd->ijab", g[V, V, V, V], t2)
    r2 -= ein("kbcj,ikca->ijab", g[O, V, V, O], t2)
    r2 += ein("kaci,kjcb->ijab", 2.0 * g[O, V, V, O] - gx[O, V, V, O], t2)
    r2 -= ein("kbic,kjac->ijab", g[O, V, O, V], t2)
    r2 -= ein("kaci,kjbc->ijab", g[O, V, V, O], t2)
    r2 += ein("kbcj,ikac->ijab", 2.0 * g[O, V, V, O] - gx[O, V, V, O], t2)
    r2 -= ein("kajc,ikcb->ijab", g[O, V, O, V], t2)
    r2 -= E * t2
    return r1, r2


def cid_spatial_residual(F, ERI_MO, t2, E, no: int):
    """The closed-shell CID residual in the reference's own symmetrised form,
    apyib/ci_wfn.py:84-95 (half the terms, then r + r with (i,a) <-> (j,b) swapped)."""
    O, V = slice(0, no), slice(no, F.shape[0])
    g = ERI_MO.swapaxes(1, 2)
    ein = lambda s, *a: np.einsum(s, *a, optimize=True)
    r2 = 0.5 * g.swapaxes(0, 2).swapaxes(1, 3)[O, O, V, V]
    r2 = r2 + ein("ijae,be->ijab", t2, F[V, V])
    r2 -= ein("imab,mj->ijab", t2, F[O, O])
    r2 += 0.5 * ein("mnab,mnij->ijab", t2, g[O, O, O, O])
    r2 += 0.5 * ein("ijef,abef->ijab", t2, g[V, V, V, V])
    r2 += ein("imae,mbej->ijab", t2 - t2.swapaxes(2, 3), g[O, V, V, O])
    r2 += ein("imae,mbej->ijab", t2, g[O, V, V, O] - g.swapaxes(2, 3)[O, V, V, O])
    r2 -= ein("mjae,mbie->ijab", t2, g[O, V, O, V])
    r2 = r2 + r2.swapaxes(0, 1).swapaxes(2, 3)
    return r2 - E * t2


def so_denominators(eps_o_spatial, eps_v_spatial):
    """apyib/ci_wfn.py:268-271: SO denominators from np.repeat-ed spatial energies."""
    eo = np.repeat(eps_o_spatial, 2)
    ev = np.repeat(eps_v_spatial, 2)
    D_ia = eo.reshape(-1, 1) - ev
    D_ijab = eo.reshape(-1, 1, 1, 1) + eo.reshape(-1, 1, 1) - ev.reshape(-1, 1) - ev
    return D_ia, D_ijab


def solve_cisd_so(F, blk, eps_o, eps_v, params, singles=True, history=None):
    """apyib/ci_wfn.py:263-378 (singles=True) and :171-259 (CID_SO).
    Returns (E, t1, t2) for CISD_SO and (E, t2) for CID_SO (t1 is None).
    ``history`` (a list) receives one dict per iteration."""
    o = 2 * len(eps_o)
    D_ia, D_ijab = so_denominators(eps_o, eps_v)
    O = slice(0, o)
    V = slice(o, F.shape[0])
    oovv = blk["oovv"]
    t2 = blk["vvoo"].transpose(2, 3, 0, 1) / D_ijab
    if singles:
        t1 = F.T[O, V] / D_ia
        E = np.einsum("ia,ia->", t1, F[O, V]) + 0.25 * np.einsum("ijab,ijab->", t2, oovv)
    else:
        t1 = None
        E = 0.25 * np.einsum("ijab,ijab->", t2, oovv)
    t1 = None if t1 is None else t1.copy()
    t2 = t2.copy()
    n1 = 0 if t1 is None else t1.size
    it = 1
    e_iter = t_iter = None
    while it <= params["max_iterations"]:
        E_old = E
        t1_old = None if t1 is None else t1.copy()
        t2_old = t2.copy()
        r1, r2 = cisd_so_residual(F, blk, t1, t2, E, o, singles)
        if singles:
            t1 = t1 + r1 / D_ia
        t2 = t2 + r2 / D_ijab
        if params["DIIS"]:
            res = r2.reshape(-1) if not singles else np.concatenate((r1.reshape(-1), r2.reshape(-1)))
            tv = t2.reshape(-1) if not singles else np.concatenate((t1.reshape(-1), t2.reshape(-1)))
            if it == 1:
                t_iter = tv.reshape(-1, 1)
                e_iter = res.reshape(-1, 1)
            tv, e_iter, t_iter = solve_general_DIIS(res, tv, e_iter, t_iter, it)
            if singles:
                t1 = tv[:n1].reshape(t1.shape)
            t2 = tv[n1:].reshape(t2.shape)
        if singles:
            E = np.einsum("ia,ia->", t1, F[O, V]) + 0.25 * np.einsum("ijab,ijab->", t2, oovv)
        else:
            E = 0.25 * np.einsum("ijab,ijab->", oovv, t2)
        d2 = t2_old - t2
        rms_t2 = np.sqrt(np.einsum("ijab,ijab->", d2, d2))
        if singles:
            d1 = t1_old - t1
            rms_t1 = np.sqrt(np.einsum("ia,ia->", d1, d1))
        else:
            rms_t1 = 0.0
        dE = E_old - E
        if history is not None:
            history.append(dict(iteration=it, E=E, dE=dE, rms_t1=rms_t1, rms_t2=rms_t2))
        if it > 1:
            ok = abs(dE) < params["e_convergence"] and rms_t2 < params["d_convergence"]
            if singles:
                ok = ok and rms_t1 < params["d_convergence"]
            if ok:
                break
        it += 1
    if singles:
        return E, t1, t2
    return E, t2


def solve_mp2_so(blk, eps_o, eps_v):
    """apyib/mp2_wfn.py:64-87: t2 = <ij||ab>-form amplitudes / D, E = 1/4 sum <ij||ab> t2."""
    _, D_ijab = so_denominators(eps_o, eps_v)
    t2 = blk["vvoo"].transpose(2, 3, 0, 1) / D_ijab
    E = 0.25 * np.einsum("ijab,ijab->", blk["oovv"], t2)
    return E, t2


def solve_mp2_spatial(ERI_MO, eps_o, eps_v):
    """apyib/mp2_wfn.py:42-59: t2 = <ab|ij>/D, E = sum (2<ij|ab> - <ij|ba>) t2 over
    spatial orbitals; ERI_MO is the active chemist tensor, occupied orbitals first."""
    no = len(eps_o)
    O = slice(0, no)
    V = slice(no, ERI_MO.shape[0])
    dirac = ERI_MO.transpose(0, 2, 1, 3)
    D = eps_o.reshape(-1, 1, 1, 1) + eps_o.reshape(-1, 1, 1) - eps_v.reshape(-1, 1) - eps_v
    t2 = dirac[V, V, O, O].transpose(2, 3, 0, 1) / D
    E = np.einsum("ijab,ijab->", 2 * dirac[O, O, V, V] - dirac[O, O, V, V].transpose(0, 1, 3, 2), t2)
    return E, t2


# ----------------------------------------------------------------------------
# AO -> MO, Fock and SCF
# ----------------------------------------------------------------------------


def compute_ERI_MO(ERI_AO, C):
    """apyib/utils.py:258-279, four quarter steps over the active columns C."""
    X = np.einsum("mnlg,gs->mnls", ERI_AO, C, optimize=True)
    X = np.einsum("mnls,lr->mnrs", X, C.conj(), optimize=True)
    X = np.einsum("nq,mnrs->mqrs", C, X, optimize=True)
    return np.einsum("mp,mqrs->pqrs", C.conj(), X, optimize=True)


def jk_fock(h, ERI_AO, D, scale=1.0):
    """F = h + scale * sum_ls D_ls (2 (mn|ls) - (ml|ns)); apyib/hf_wfn.py:81
    (scale 0.5, D = 2 C_o C_o^*) and apyib/utils.py:249 (scale 1, D = C_o C_o^*)."""
    J = np.einsum("ls,mnls->mn", D, ERI_AO, optimize=True)
    K = np.einsum("ls,mlns->mn", D, ERI_AO, optimize=True)
    return h + scale * (2 * J - K)


def compute_F_MO(h_AO, ERI_AO, C, nfzc, ndocc, nbf, freeze_core=False):
    """apyib/utils.py:217-254."""
    f = slice(0, nfzc)
    o = slice(nfzc, ndocc)
    t = slice(nfzc, nbf)
    E_fc = 0
    if freeze_core:
        D_fc = C[:, f] @ C[:, f].conj().T
        h_fc = jk_fock(h_AO, ERI_AO, D_fc)
        E_fc = np.einsum("nm,mn->", D_fc, h_AO + h_fc)
        h_AO = h_fc
    D = C[:, o] @ C[:, o].conj().T
    F_AO = jk_fock(h_AO, ERI_AO, D)
    F_MO = C[:, t].conj().T @ F_AO @ C[:, t]
    return F_MO, E_fc


def solve_scf(T, V, S, ERI, E_nuc, ndocc, params, history=None):
    """apyib/hf_wfn.py:36-170.  Returns (E_SCF, C, eps)."""
    import scipy.linalg as la

    nbf = S.shape[0]
    H_core = T + V
    X = np.linalg.inv(la.sqrtm(S))
    F_p = X @ H_core @ X
    e, C_p = np.linalg.eigh(F_p)
    C = X @ C_p
    eps = np.zeros(nbf)
    Cc = np.zeros((nbf, nbf))
    D = 2 * C[:, :ndocc] @ C[:, :ndocc].conj().T
    E_SCF = np.sum(0.5 * D * (H_core + H_core))
    i = 1
    e_iter = F_iter = None
    while i <= params["max_iterations"]:
        E_old = E_SCF
        D_old = D
        F = jk_fock(H_core, ERI, D, 0.5)
        if params["DIIS"]:
            SDF = S @ D @ F
            res = (X @ (SDF - SDF.conj().T) @ X).reshape(-1)
            Fv = F.reshape(-1)
            if i == 1:
                F_iter = Fv.reshape(-1, 1)
                e_iter = res.reshape(-1, 1)
            Fv, e_iter, F_iter = solve_general_DIIS(res, Fv, e_iter, F_iter, i)
            F = Fv.reshape(nbf, nbf)
        F_p = X @ F @ X
        eps, C_p = np.linalg.eigh(F_p)
        C = Cc = X @ C_p
        D = 2 * C[:, :ndocc] @ C[:, :ndocc].conj().T
        E_SCF = np.sum(0.5 * D.T * (H_core + F))
        dE = E_SCF - E_old
        rms_D = np.sqrt(np.sum((D_old - D) ** 2))
        if history is not None:
            history.append(dict(iteration=i, E=E_SCF, dE=dE, rms_D=rms_D))
        if i > 1 and abs(dE) < params["e_convergence"] and rms_D < params["d_convergence"]:
            break
        i += 1
    return E_SCF, Cc, eps


# ----------------------------------------------------------------------------
# Adjoint reference: one- and two-particle densities
# ----------------------------------------------------------------------------


def cisd_so_densities(t1, t2, o, n):
    """Normalised OPD/TPD of the CISD_SO wavefunction, restating the adjoint
    check kept (commented) in apyib/ci_wfn.py:382-411:
    E_corr + E_ref-terms = sum F_pq D_pq + sum <pq|rs> D_pqrs."""
    O = slice(0, o)
    V = slice(o, n)
    cj = np.conjugate
    ein = lambda s, *a: np.einsum(s, *a, optimize=True)
    N = 1 / np.sqrt(1 + ein("ia,ia->", cj(t1), t1) + 0.25 * ein("ijab,ijab->", cj(t2), t2))
    t0 = N
    t1 = t1 * N
    t2 = t2 * N
    D = np.zeros((n, n), dtype=complex)
    D[O, O] -= ein("ja,ia->ij", cj(t1), t1) + 0.5 * ein("jkab,ikab->ij", cj(t2), t2)
    D[V, V] += ein("ia,ib->ab", cj(t1), t1) + 0.5 * ein("ijac,ijbc->ab", cj(t2), t2)
    D[O, V] += cj(t0) * t1 + ein("jb,ijab->ia", cj(t1), t2)
    D[V, O] += cj(t1.T) * t0 + ein("ijab,jb->ai", cj(t2), t1)
    G = np.zeros((n, n, n, n), dtype=complex)
    G[O, O, O, O] += 0.25 * ein("klab,ijab->ijkl", cj(t2), t2)
    G[V, V, V, V] += 0.25 * ein("ijab,ijcd->abcd", cj(t2), t2)
    G[O, V, V, O] += ein("ja,ib->iabj", cj(t1), t1)
    G[O, V, O, V] -= ein("ja,ib->iajb", cj(t1), t1)
    G[V, O, O, V] += ein("jkac,ikbc->aijb", cj(t2), t2)
    G[V, O, V, O] -= ein("jkac,ikbc->aibj", cj(t2), t2)
    G[O, O, V, V] += 0.5 * cj(t0) * t2
    G[V, V, O, O] += 0.5 * cj(t2.transpose(2, 3, 0, 1)) * t0
    G[V, O, V, V] += ein("ja,ijcb->aibc", cj(t1), t2)
    G[O, V, O, O] -= ein("kjab,ib->iajk", cj(t2), t1)
    G[V, V, V, O] += ein("jiab,jc->abci", cj(t2), t1)
    G[O, O, O, V] -= ein("kb,ijba->ijka", cj(t1), t2)
    return D, G
