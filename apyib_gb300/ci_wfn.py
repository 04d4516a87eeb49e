"""Spin-orbital CISD / CID over complex orbitals on the GPU
(drop-in for apyib/ci_wfn.py:19-416).

``parameters`` is the reference's dict; two optional keys select the
precision of the residual contractions:
  'precision': 'fp64' (default, the parity mode) or 'mixed' (3xTF32
               tensor-core residuals with FP64 defect correction);
  'switch_tol': |dE| at which the mixed solve switches to defect correction.
"""
from __future__ import annotations

import numpy as np
import torch

from .cisd import CISDPlan, solve
from .device import to_dev
from .utils import compute_ERI_MO, compute_F_MO, compute_F_SO, get_slices


class ci_wfn(object):
    def __init__(self, parameters, wfn):
        self.parameters = parameters
        self.H = wfn.H
        self.wfn = wfn
        self.C = wfn.C
        self.C_list, self.I_list = get_slices(self.parameters, self.wfn)
        o = self.C_list[1]
        v = self.C_list[2]
        self.eps_o = np.asarray(wfn.eps)[o]
        self.eps_v = np.asarray(wfn.eps)[v]
        self.D_ia = self.eps_o.reshape(-1, 1) - self.eps_v
        self.D_ijab = (self.eps_o.reshape(-1, 1, 1, 1) + self.eps_o.reshape(-1, 1, 1) - self.eps_v.reshape(-1, 1)
                       - self.eps_v)
        # MO integrals stay on the device
        self._F_MO, _ = compute_F_MO(self.parameters, self.wfn, self.C_list, return_torch=True)
        self._ERI_MO = compute_ERI_MO(self.parameters, self.wfn, self.C_list, return_torch=True)
        self.history = []

    @property
    def F_MO(self):
        return self._F_MO.cpu().numpy()

    @property
    def ERI_MO(self):
        return self._ERI_MO.cpu().numpy()

    def _plan(self, singles):
        o, v = 2 * len(self.eps_o), 2 * len(self.eps_v)
        mixed = self.parameters.get("precision", "fp64") == "mixed"
        plan = CISDPlan(o, v, singles=singles, mixed=mixed)
        F_SO = compute_F_SO(self.wfn, self._F_MO, return_torch=True)
        eps_so = np.concatenate([np.repeat(self.eps_o, 2), np.repeat(self.eps_v, 2)])
        plan.set_fock(F_SO, eps_so)
        plan.blocks_from_mo(self._ERI_MO)
        return plan

    def _solve(self, singles, print_level):
        plan = self._plan(singles)
        prec = self.parameters.get("precision", "fp64")
        self.history = []
        E, t = solve(plan, self.parameters, precision=prec, print_level=print_level, history=self.history,
                     switch_tol=self.parameters.get("switch_tol", 1e-8))
        t1, t2 = plan.unpack(t)
        return np.complex128(E), t1, t2

    def solve_CISD_SO(self, print_level=0, return_torch=False):
        """apyib/ci_wfn.py:263-416; returns (E_CISD, t1[o,v], t2[o,o,v,v])."""
        E, t1, t2 = self._solve(True, print_level)
        if return_torch:
            return E, t1, t2
        return E, t1.cpu().numpy(), t2.cpu().numpy()

    def solve_CID_SO(self, print_level=0, return_torch=False):
        """apyib/ci_wfn.py:171-259; returns (E_CID, t2[o,o,v,v])."""
        E, _, t2 = self._solve(False, print_level)
        if return_torch:
            return E, t2
        return E, t2.cpu().numpy()

    # Closed-shell spatial-orbital solvers: the reference's spin-adapted equations
    # (apyib/ci_wfn.py:51-167, 420-574) on the library's GEMMs (apyib_gb300.spatial).  With
    # parameters['precision'] = 'mixed' they run on the spin-orbital engine instead (its
    # tensor-core residuals and defect correction) and return the spatial amplitudes
    # t1[i,a] = t1_SO[2i,2a], t2[i,j,a,b] = t2_SO[2i,2j+1,2a,2b+1] (alpha-beta block).

    def _solve_spatial(self, singles, print_level):
        from .spatial import SpatialCISD
        no = len(self.eps_o)
        eng = SpatialCISD(self._F_MO, self._ERI_MO, no, singles=singles)
        eng.set_denominators(self.eps_o, self.eps_v)
        self.history = []
        E, t1, t2 = eng.solve(self.parameters, print_level=print_level, history=self.history)
        return np.complex128(E), t1, t2

    def solve_CISD(self, print_level=0, return_torch=False):
        """apyib/ci_wfn.py:420-574; returns (E_CISD, t1[no,nv], t2[no,no,nv,nv])."""
        if self.parameters.get("precision", "fp64") == "mixed":
            E, t1, t2 = self._solve(True, print_level)
            t1s = t1[0::2, 0::2].contiguous()
            t2s = t2[0::2, 1::2, 0::2, 1::2].contiguous()
        else:
            E, t1s, t2s = self._solve_spatial(True, print_level)
        if return_torch:
            return E, t1s, t2s
        return E, t1s.cpu().numpy(), t2s.cpu().numpy()

    def solve_CID(self, print_level=0, return_torch=False):
        """apyib/ci_wfn.py:51-167; returns (E_CID, t2[no,no,nv,nv])."""
        if self.parameters.get("precision", "fp64") == "mixed":
            E, _, t2 = self._solve(False, print_level)
            t2s = t2[0::2, 1::2, 0::2, 1::2].contiguous()
        else:
            E, _, t2s = self._solve_spatial(False, print_level)
        if return_torch:
            return E, t2s
        return E, t2s.cpu().numpy()


def solve_so_system(F_SO, eps_o, eps_v, params, B=None, ERI_SO=None, singles=True, precision="fp64",
                    print_level=0, history=None, return_plan=False):
    """CISD_SO / CID_SO for a spin-orbital system given directly (F_SO, the
    spatial orbital energies whose np.repeat gives the SO denominators, and
    either Hermitian factors B[L,p,q] or a full chemist ERI_SO) - the entry
    the synthetic workloads use, equivalent to calling solve_CISD_SO with
    compute_F_SO / compute_ERI_SO returning these tensors."""
    o, v = 2 * len(eps_o), 2 * len(eps_v)
    plan = CISDPlan(o, v, singles=singles, mixed=(precision == "mixed"))
    eps_so = np.concatenate([np.repeat(eps_o, 2), np.repeat(eps_v, 2)])
    plan.set_fock(to_dev(F_SO), eps_so)
    if B is not None:
        plan.blocks_from_factors(to_dev(B))
    else:
        plan.blocks_from_so(to_dev(ERI_SO))
    E, t = solve(plan, params, precision=precision, print_level=print_level, history=history)
    if return_plan:
        return np.complex128(E), t, plan
    t1, t2 = plan.unpack(t)
    return np.complex128(E), t1, t2
