"""MP2 in spin orbitals over complex orbitals (drop-in for apyib/mp2_wfn.py:16-87)."""
from __future__ import annotations

import numpy as np

from . import _lib
from .cisd import CISDPlan
from .device import to_dev
from .utils import compute_ERI_MO, get_slices


class mp2_wfn(object):
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
        self.D_ijab = (self.eps_o.reshape(-1, 1, 1, 1) + self.eps_o.reshape(-1, 1, 1) - self.eps_v.reshape(-1, 1)
                       - self.eps_v)

    def solve_MP2(self, return_torch=False):
        """apyib/mp2_wfn.py:42-59: closed-shell MP2 over complex spatial orbitals on the GPU."""
        import ctypes

        import torch

        from .device import ptr, stream_ptr
        ERI_MO = compute_ERI_MO(self.parameters, self.wfn, self.C_list, return_torch=True)
        no, nv = len(self.eps_o), len(self.eps_v)
        nmo = no + nv
        eps = to_dev(np.concatenate([self.eps_o, self.eps_v]), torch.float64)
        t2 = torch.empty((no, no, nv, nv), dtype=torch.complex128, device=ERI_MO.device)
        E = torch.empty(1, dtype=torch.complex128, device=ERI_MO.device)
        part = torch.empty(1024, dtype=torch.complex128, device=ERI_MO.device)
        _lib.call("agb_mp2_spatial", ptr(ERI_MO), nmo, no, ptr(eps), ptr(t2), ptr(E), ptr(part),
                  ctypes.c_size_t(part.numel() * 16), stream_ptr())
        Ev = np.complex128(E.cpu().numpy()[0])
        return (Ev, t2) if return_torch else (Ev, t2.cpu().numpy())

    def solve_MP2_SO(self, return_torch=False):
        """apyib/mp2_wfn.py:64-87: t2 = <ij||ab>/D, E = 1/4 sum <ij||ab> t2, on the GPU."""
        ERI_MO = compute_ERI_MO(self.parameters, self.wfn, self.C_list, return_torch=True)
        o, v = 2 * len(self.eps_o), 2 * len(self.eps_v)
        plan = CISDPlan(o, v, mp2_only=True)
        eps_so = np.concatenate([np.repeat(self.eps_o, 2), np.repeat(self.eps_v, 2)])
        import torch
        F_dummy = torch.diag(to_dev(eps_so))   # MP2 reads only the denominators
        plan.set_fock(F_dummy, eps_so)
        plan.blocks_from_mo(ERI_MO)
        E, t = plan.mp2()
        _, t2 = plan.unpack(t)
        if return_torch:
            return np.complex128(E), t2
        return np.complex128(E), t2.cpu().numpy()
