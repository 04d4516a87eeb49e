"""Generate ``c3res_40_160.npz``: one CISD_SO iteration of the UNMODIFIED
reference (apyib/ci_wfn.py:263-337, loaded by ``ref_loader`` with a stub psi4)
at o/v = 40/160 spin orbitals, nso = 200, naux = 800 — the residual-scale
parity case at the size class of the o/v = 40/160 workload.

The reference needs the full nso^4 ERI_SO (25.6 GB) only through
``swapaxes``, ``copy`` and 4-slice indexing, so a lazy stand-in supplies it:
each requested block is formed from the seeded Hermitian factors,
(pq|rs) = sum_L B_L[p,q] B_L[r,s], when the reference slices it (the two most
recent blocks are kept).  A non-diagonal complex Fock matrix makes every Fock
term of the residual count.  With max_iterations=1 and no DIIS the returned
amplitudes are t_1 = t_0 + r(t_0)/D (apyib/ci_wfn.py:336-337).

Stored (small): the seed and an input digest, t1 after the iteration (o*v),
the energy, 4096 probes of t2 at seeded random (i,j,a,b), and three seeded
random projections sum_ijab w_ijab t2_ijab.  Inputs are regenerated from the
seed by apyib_gb300.synthetic on both sides.

Run from the repository root where the reference sources are available
(about 5 minutes and 35 GB of host memory on 8 cores):

    APYIB_REF=/path/to/apyib python tests/golden/make_golden_c3.py
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_loader  # noqa: E402
from apyib_gb300 import synthetic  # noqa: E402
from c3_case import FIXTURE, NPROBE, O, SEED, V, digest, perturbed_fock, probe_indices, projection_weights  # noqa: E402
from make_golden import fake_hamiltonian, params  # noqa: E402


class LazyERI:
    """Chemist ERI_SO stand-in: a permutation of the chemist axes plus a small
    block cache; ``swapaxes`` permutes, ``copy`` returns the same immutable
    object, and a 4-slice index forms that block from the factors."""

    def __init__(self, B, perm=(0, 1, 2, 3), cache=None):
        self.B = B
        self.perm = perm
        self.cache = cache if cache is not None else {}
        n = B.shape[1]
        self.shape = (n, n, n, n)

    def swapaxes(self, a, b):
        p = list(self.perm)
        p[a], p[b] = p[b], p[a]
        return LazyERI(self.B, tuple(p), self.cache)

    def copy(self):
        return self

    def __getitem__(self, key):
        chem = [None] * 4
        for k in range(4):
            chem[self.perm[k]] = key[k]
        ck = tuple((s.start, s.stop, s.step) for s in chem)
        if ck not in self.cache:
            while len(self.cache) >= 2:
                self.cache.pop(next(iter(self.cache)))
            P, Q, R, S = chem
            Bl, Br = self.B[:, P, Q], self.B[:, R, S]
            L = Bl.shape[0]
            blk = (Bl.reshape(L, -1).T @ Br.reshape(L, -1)).reshape(Bl.shape[1:] + Br.shape[1:])
            self.cache[ck] = blk
        return self.cache[ck].transpose(self.perm)


def main():
    ref = ref_loader.load_reference()
    prob = synthetic.so_factors(O, V, seed=SEED)
    Fp = perturbed_fock(prob, O, V, SEED)
    nbf = (O + V) // 2
    wfn = types.SimpleNamespace(H=fake_hamiltonian(nbf), nbf=nbf, ndocc=O // 2,
                                eps=np.concatenate([prob.eps_o, prob.eps_v]), C=np.eye(nbf), E_SCF=0.0)
    ci = ref.ci_wfn
    saved = {k: getattr(ci, k) for k in ("compute_F_MO", "compute_ERI_MO", "compute_F_SO", "compute_ERI_SO")}
    try:
        ci.compute_F_MO = lambda p, w, c: (None, 0)
        ci.compute_ERI_MO = lambda p, w, c: None
        ci.compute_F_SO = lambda w, f: Fp
        ci.compute_ERI_SO = lambda w, e: LazyERI(prob.B)
        E1, t1, t2 = ci.ci_wfn(params("CISD_SO", maxit=1, diis=False), wfn).solve_CISD_SO()
    finally:
        for k, f in saved.items():
            setattr(ci, k, f)
    idx = probe_indices(O, V, NPROBE, SEED + 1)
    proj = np.array([np.sum(projection_weights(O, V, SEED + 2 + k) * t2) for k in range(3)])
    out = dict(o=O, v=V, seed=SEED, input_sha=digest(prob.B, prob.eps_o, prob.eps_v, Fp),
               E_iter1=E1, t1_iter1=t1, probe_idx=idx, t2_probes=t2[idx[0], idx[1], idx[2], idx[3]],
               t2_proj=proj, t2_norm2=np.sum(np.abs(t2) ** 2))
    np.savez_compressed(os.path.join(HERE, FIXTURE), **out)
    print("c3", E1, proj)


if __name__ == "__main__":
    main()
