"""Analytic atomic polar tensors of RHF at zero field (apyib/analytic_apts.py interface).

* Length gauge (``compute_RHF_APTs_LG``): d mu / dR from analytic nuclear gradients
  in +- electric field (gradient.apt).
* Velocity gauge (``compute_RHF_APTs_VG``, the quantity of apyib/analytic_apts.py:
  190-385): the perturbation is the imaginary velocity operator with MO elements
  i <p| d/dr |q> (the nabla integrals), whose closed-shell CPHF response U^E has
  the structure of the magnetic one; the electronic part is then
  -2 Im d^2 <Phi(R) | Phi(E)> / dR dE over the linearised determinants (the
  overlap derivative analytic_aats evaluates for the AATs) and the nuclear charges
  add Z delta.
"""
from __future__ import annotations

import numpy as np
import torch

from .analytic_aats import _mo
from .analytic_aats import analytic_derivative as _aat_derivative
from .gradient import apt as _apt
from .linalg import cg_solve


class analytic_derivative(_aat_derivative):
    def compute_RHF_APTs_LG(self, orbitals="non-canonical"):
        return _apt(dict(self.parameters, method="RHF"))

    def compute_RHF_APTs_VG(self, orbitals="non-canonical"):
        from .integrals import MintsHelper
        self._setup()
        nbf, no, Cc = self.nbf, self.no, self.Cc
        nv = nbf - no
        v, o = slice(no, nbf), slice(0, no)
        nab = MintsHelper(self.H.basis_set).ao_nabla(return_torch=True)
        UE, hE, rhs = [], [], []
        for b in range(3):
            Y = _mo(Cc, nab[b])                                  # h^E = i Y, Y = <p| d/dr_b |q>
            hE.append(1j * Y)
            rhs.append(-Y[v, o].reshape(-1))
        X = cg_solve(self.Am, torch.stack(rhs, dim=1))
        for b in range(3):
            U = torch.zeros((nbf, nbf), dtype=torch.complex128, device=Cc.device)
            U[v, o] = 1j * X[:, b].reshape(nv, no)
            U[o, v] = 1j * X[:, b].reshape(nv, no).T
            UE.append(U)
        self.UB, self.hB = UE, hE
        I = self._aats("RHF", "intermediate", setup=False)
        Z = self.H.molecule.Z.astype(float)
        N = np.zeros((3 * len(Z), 3))
        for k in range(3 * len(Z)):
            N[k, k % 3] = Z[k // 3]
        return -2.0 * I + N
