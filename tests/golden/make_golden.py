"""Generate the golden fixtures in this directory by running the UNMODIFIED
reference apyib hot-path modules (loaded by ``ref_loader`` with a stub psi4)
on seeded synthetic inputs.

Run from the repository root where the reference sources are available:

    APYIB_REF=/path/to/apyib python tests/golden/make_golden.py

Outputs (small .npz files, committed):
  so_<o>_<v>_<kind>.npz   spin-orbital CISD_SO / CID_SO / MP2_SO solves and a
                          single-residual evaluation, inputs stored when small
  ao_<nbf>_<field>.npz    SCF -> F_MO/ERI_MO -> SO expansion -> CISD_SO/MP2_SO
                          from a synthetic AO problem, plus one DIIS call
The reference functions exercised are apyib/ci_wfn.py:24-47,171-259,263-416,
apyib/mp2_wfn.py:21-39,64-87, apyib/hf_wfn.py:14-170 and
apyib/utils.py:104-140,184-365.
"""
import hashlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_loader  # noqa: E402
from apyib_gb300 import synthetic  # noqa: E402

ref = ref_loader.load_reference()


def digest(*arrs):
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def fake_hamiltonian(nbf, nfzc=0, ao=None, E_nuc=0.0, nelec=None):
    basis = types.SimpleNamespace(nbf=lambda: nbf, n_frozen_core=lambda: nfzc)
    # A molecule whose atomic numbers sum to nelec (hf_wfn.nelectron, apyib/hf_wfn.py:28-33).
    mol = types.SimpleNamespace(natom=lambda: 1, true_atomic_number=lambda a: nelec)
    H = types.SimpleNamespace(basis_set=basis, molecule=mol, E_nuc=E_nuc)
    if ao is not None:
        H.S, H.T, H.V, H.ERI = ao.S, ao.T, ao.V, ao.ERI
    return H


def params(method, maxit=100, diis=True, fc=False, econv=1e-13, dconv=1e-13):
    return dict(method=method, e_convergence=econv, d_convergence=dconv, DIIS=diis,
                freeze_core=fc, max_iterations=maxit, F_el=[0, 0, 0], F_mag=[0, 0, 0])


def so_case(o, v, seed, real=False, store_inputs=True):
    prob = synthetic.so_factors(o, v, seed=seed, real=real)
    B = prob.B
    eri = np.einsum("Lpq,Lrs->pqrs", B, B, optimize=True)   # chemist SO tensor
    F_SO = prob.fock_so()
    nbf = (o + v) // 2
    H = fake_hamiltonian(nbf)
    wfn = types.SimpleNamespace(H=H, nbf=nbf, ndocc=o // 2, eps=np.concatenate([prob.eps_o, prob.eps_v]),
                                C=np.eye(nbf), E_SCF=0.0)
    out = dict(o=o, v=v, seed=seed, real=int(real), input_sha=digest(B, prob.eps_o, prob.eps_v))
    if store_inputs:
        out.update(B=B, eps_o=prob.eps_o, eps_v=prob.eps_v)
    ci = ref.ci_wfn
    mp = ref.mp2_wfn
    saved = {m: {k: getattr(m, k) for k in ("compute_F_MO", "compute_ERI_MO", "compute_F_SO", "compute_ERI_SO")}
             for m in (ci, mp)}
    try:
        for m in (ci, mp):
            m.compute_F_MO = lambda p, w, c: (None, 0)
            m.compute_ERI_MO = lambda p, w, c: None
            m.compute_F_SO = lambda w, f: F_SO
            m.compute_ERI_SO = lambda w, e: eri
        E, t1, t2 = ci.ci_wfn(params("CISD_SO"), wfn).solve_CISD_SO()
        out.update(E_cisd=E, t1_cisd=t1, t2_cisd=t2)
        E, t2 = ci.ci_wfn(params("CID_SO"), wfn).solve_CID_SO()
        out.update(E_cid=E, t2_cid=t2)
        E, t2 = mp.mp2_wfn(params("MP2_SO"), wfn).solve_MP2_SO()
        out.update(E_mp2=E, t2_mp2=t2)
        # One iteration without DIIS from a perturbed guess recovers the residual:
        # r = (t_after - t_before) * D (apyib/ci_wfn.py:336-337).  A non-diagonal
        # F_SO makes every Fock term of the residual count.
        rng = np.random.default_rng(seed + 1000)
        Fp = F_SO.copy()
        pert = (rng.standard_normal(F_SO.shape) + 1j * rng.standard_normal(F_SO.shape)) * 0.01
        pert = pert + pert.conj().T
        mask = np.add.outer(np.arange(o + v) % 2, np.arange(o + v) % 2) % 2 == 0
        Fp = Fp + pert * mask
        for m in (ci,):
            m.compute_F_SO = lambda w, f: Fp
        E1, t1_1, t2_1 = ci.ci_wfn(params("CISD_SO", maxit=1, diis=False), wfn).solve_CISD_SO()
        out.update(F_pert=Fp, E_iter1=E1, t1_iter1=t1_1, t2_iter1=t2_1)
    finally:
        for m, d in saved.items():
            for k, f in d.items():
                setattr(m, k, f)
    return out


def ao_case(nbf, ndocc, seed, field, nfzc=0):
    ao = synthetic.ao_problem(nbf, ndocc, seed=seed, field=field, nfzc=nfzc)
    H = fake_hamiltonian(nbf, nfzc=nfzc, ao=ao, E_nuc=ao.E_nuc, nelec=2 * ndocc)
    out = dict(nbf=nbf, ndocc=ndocc, seed=seed, field=field, nfzc=nfzc,
               S=ao.S, T=ao.T, V=ao.V, ERI=ao.ERI, E_nuc=ao.E_nuc)
    wfn = ref.hf_wfn.hf_wfn(H)
    E_SCF, C = wfn.solve_SCF(params("RHF", fc=nfzc > 0))
    out.update(E_scf=E_SCF, C=C, eps=wfn.eps)
    for method in ("CISD_SO", "MP2_SO"):
        p = params(method, fc=nfzc > 0)
        C_list, I_list = ref.utils.get_slices(p, wfn)
        if method == "CISD_SO":
            F_MO, E_fc = ref.utils.compute_F_MO(p, wfn, C_list)
            ERI_MO = ref.utils.compute_ERI_MO(p, wfn, C_list)
            out.update(F_MO=F_MO, E_fc=E_fc, ERI_MO=ERI_MO)
            w = ref.ci_wfn.ci_wfn(p, wfn)
            E, t1, t2 = w.solve_CISD_SO()
            out.update(E_cisd=E, t1_cisd=t1, t2_cisd=t2)
            E, t2 = ref.ci_wfn.ci_wfn(params("CID_SO", fc=nfzc > 0), wfn).solve_CID_SO()
            out.update(E_cid=E)
            # closed-shell spatial solvers (apyib/ci_wfn.py:51-167, 420-574)
            import contextlib
            import io
            with contextlib.redirect_stdout(io.StringIO()):
                E, t1, t2 = ref.ci_wfn.ci_wfn(params("CISD", fc=nfzc > 0), wfn).solve_CISD()
                out.update(E_cisd_spatial=E, t1_cisd_spatial=t1, t2_cisd_spatial=t2)
                E, t2 = ref.ci_wfn.ci_wfn(params("CID", fc=nfzc > 0), wfn).solve_CID()
                out.update(E_cid_spatial=E, t2_cid_spatial=t2)
        else:
            E, t2 = ref.mp2_wfn.mp2_wfn(p, wfn).solve_MP2_SO()
            out.update(E_mp2=E, t2_mp2=t2)
            E, t2 = ref.mp2_wfn.mp2_wfn(params("MP2", fc=nfzc > 0), wfn).solve_MP2()
            out.update(E_mp2_spatial=E, t2_mp2_spatial=t2)
    return out


def diis_case(seed):
    rng = np.random.default_rng(seed)
    n = 37
    out = dict(seed=seed)
    e_iter = t_iter = None
    vecs = []
    for it in range(1, 11):
        r = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        t = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        r *= 0.5 ** it
        if it == 1:
            t_iter = np.atleast_2d(t).T
            e_iter = np.atleast_2d(r).T
        tv, e_iter, t_iter = ref.utils.solve_general_DIIS({}, r, t, e_iter, t_iter, it)
        vecs.append((r, t, tv))
    out["r"] = np.array([a for a, _, _ in vecs])
    out["t"] = np.array([b for _, b, _ in vecs])
    out["tv"] = np.array([c for _, _, c in vecs])
    return out


def main():
    np.savez_compressed(os.path.join(HERE, "diis.npz"), **diis_case(7))
    for (o, v, seed, real, store) in [(2, 4, 1, False, True), (4, 6, 2, False, True), (4, 6, 3, True, True),
                                      (6, 10, 4, False, True), (10, 38, 5, False, False)]:
        d = so_case(o, v, seed, real, store)
        if not store:
            for k in ("t2_cisd", "t2_cid", "t2_mp2", "t2_iter1", "F_pert"):
                d.pop(k, None)
        np.savez_compressed(os.path.join(HERE, f"so_{o}_{v}_{'r' if real else 'c'}{seed}.npz"), **d)
        print("so", o, v, d["E_cisd"], d["E_cid"], d["E_mp2"])
    for (nbf, ndocc, seed, field, nfzc) in [(7, 3, 11, 0.0, 0), (8, 3, 12, 1e-2, 0), (9, 4, 13, 1e-2, 1)]:
        d = ao_case(nbf, ndocc, seed, field, nfzc)
        np.savez_compressed(os.path.join(HERE, f"ao_{nbf}_{ndocc}_{nfzc}_{'f' if field else 'z'}.npz"), **d)
        print("ao", nbf, d["E_scf"], d["E_cisd"], d["E_mp2"])


if __name__ == "__main__":
    main()
