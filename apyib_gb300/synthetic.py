"""Seeded synthetic inputs with the shapes of the CISD/MP2 workloads.

Two families:

* ``so_factors``: spin-orbital problems given directly by Hermitian factor
  tensors B[L,p,q] (complex), with chemist ERIs
  (pq|rs) = sum_L B[L,p,q] conj(B[L,s,r]) = sum_L B[L,p,q] B[L,r,s],
  naux = 4*nso, and a diagonal Fock matrix built from per-spatial-orbital
  energies (occupied U[-1.5,-0.3], virtual U[0.2,3.0]) duplicated into the
  interleaved alpha/beta spin orbitals, the form the reference's
  ``np.repeat`` denominators require (apyib/ci_wfn.py:268-271).
  B = (X + X^H) / 2 / sqrt(nso*naux) with X complex standard normal.  The
  1/sqrt(nso*naux) scale keeps exchange integrals K_pq = sum_L |B_pq|^2 at
  1/nso; with 1/sqrt(nso) they are naux/nso = 4 Eh and the reference's own
  Jacobi+DIIS CISD iteration diverges at every size tried.

* ``ao_problem``: a small closed-shell "molecule" in a non-orthogonal real
  AO basis (S, T+V, real 8-fold-symmetric ERIs from real factors) with an
  optional imaginary magnetic-field term i*(B.L)/2 added to the core
  Hamiltonian, as apyib/hamiltonian.py:55-70 does with mu_mag = -i/2 L.

Everything is NumPy on the host so the same seed yields the same arrays for
the GPU path and for the CPU oracle.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class SOProblem:
    o: int                # occupied spin orbitals
    v: int                # virtual spin orbitals
    B: np.ndarray         # [naux, nso, nso] complex128, Hermitian in (p,q)
    eps_o: np.ndarray     # [o/2] spatial occupied energies
    eps_v: np.ndarray     # [v/2] spatial virtual energies

    @property
    def nso(self):
        return self.o + self.v

    @property
    def naux(self):
        return self.B.shape[0]

    def fock_so(self):
        eps = np.repeat(np.concatenate([self.eps_o, self.eps_v]), 2)
        return np.diag(eps).astype(np.complex128)


def so_factors(o: int, v: int, seed: int = 0, naux: int | None = None, real: bool = False) -> SOProblem:
    """Synthetic spin-orbital CISD/MP2 problem with o occupied and v virtual
    spin orbitals (both even)."""
    if o % 2 or v % 2:
        raise ValueError("o and v count spin orbitals and must be even")
    rng = np.random.default_rng(seed)
    nso = o + v
    naux = 4 * nso if naux is None else naux
    if real:
        X = rng.standard_normal((naux, nso, nso)) * np.sqrt(2.0)
        B = (X + X.transpose(0, 2, 1)) / 2
    else:
        X = rng.standard_normal((naux, nso, nso)) + 1j * rng.standard_normal((naux, nso, nso))
        B = (X + np.conj(X.transpose(0, 2, 1))) / 2
    B = (B / np.sqrt(nso * naux)).astype(np.complex128)
    eps_o = np.sort(rng.uniform(-1.5, -0.3, o // 2))
    eps_v = np.sort(rng.uniform(0.2, 3.0, v // 2))
    return SOProblem(o, v, B, eps_o, eps_v)


@dataclasses.dataclass
class AOProblem:
    nbf: int
    ndocc: int
    S: np.ndarray        # [nbf,nbf] real symmetric positive definite
    T: np.ndarray        # [nbf,nbf] kinetic (real)
    V: np.ndarray        # [nbf,nbf] potential (complex when a field is on)
    ERI: np.ndarray      # [nbf]*4 real chemist (mn|ls), 8-fold symmetric
    E_nuc: float
    nfzc: int = 0


def ao_problem(nbf: int, ndocc: int, seed: int = 0, field: float = 0.0, naux: int | None = None,
               nfzc: int = 0) -> AOProblem:
    """Synthetic real-AO closed-shell problem.  ``field`` adds the imaginary
    Hermitian term i*field*L_z/2 (L_z real antisymmetric) to V."""
    rng = np.random.default_rng(seed)
    naux = 3 * nbf if naux is None else naux
    Q = rng.standard_normal((nbf, nbf)) * 0.08
    S = np.eye(nbf) + (Q + Q.T) / 2
    w, U = np.linalg.eigh(S)
    S = (U * np.clip(w, 0.6, None)) @ U.T
    S = (S + S.T) / 2
    T = np.diag(np.linspace(0.5, 4.0, nbf)) + 0.05 * (lambda a: a + a.T)(rng.standard_normal((nbf, nbf)))
    Vr = -np.diag(np.linspace(8.0, 1.0, nbf)) + 0.05 * (lambda a: a + a.T)(rng.standard_normal((nbf, nbf)))
    A = rng.standard_normal((naux, nbf, nbf))
    A = (A + A.transpose(0, 2, 1)) / 2 / np.sqrt(naux * nbf) * 0.5
    for L in range(naux):
        A[L] += np.eye(nbf) * (0.3 / np.sqrt(naux))
    ERI = np.einsum("Lmn,Lls->mnls", A, A, optimize=True)
    V = Vr.astype(np.complex128)
    if field != 0.0:
        Lz = rng.standard_normal((nbf, nbf))
        Lz = (Lz - Lz.T) / 2
        # mu_mag = -1/2 i L; V -= F_mag * mu_mag  =>  V += i F_mag L / 2
        V = V + 1j * field * Lz / 2
    return AOProblem(nbf, ndocc, S, T, V, ERI, E_nuc=1.2345, nfzc=nfzc)
