"""AO integrals on the GPU: the psi4 ``MintsHelper`` calls of apyib/hamiltonian.py:29-55.

``MintsHelper(basis)`` uploads the shells of a ``basis.BasisSet`` once and
evaluates, in FP64 CUDA kernels of the library (``agb_ao_one_electron``,
``agb_ao_eri``), the overlap, kinetic, nuclear-attraction, electron-repulsion,
dipole, nabla and angular-momentum integrals over the Cartesian functions;
pure (solid-harmonic) bases are then formed on the device by
``agb_ao_transform_axis``, one axis at a time.  Matrices come back as NumPy
arrays that also answer ``.np`` (the psi4 ``Matrix`` attribute the reference
reads), or as device tensors with ``return_torch=True``.

Sign conventions are psi4's, as apyib/integrals.py:143-146 restates them:
dipole integrals carry the electron charge (-<r>), angular-momentum integrals
are -<r x nabla> (real, antisymmetric; apyib/hamiltonian.py:56 multiplies them
by -i/2), nabla integrals are <d/dr> acting on the ket; origin 0 unless given.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import device, ptr, stream_ptr


class AOMatrix(np.ndarray):
    """A NumPy array that also answers ``.np`` like psi4's Matrix."""

    @property
    def np(self):
        return np.asarray(self)


def _host(t):
    return np.asarray(t.cpu().numpy()).view(AOMatrix)


class MintsHelper(object):
    def __init__(self, basis):
        self.basis = basis
        dev = device()
        flat = basis.flat()
        self._dev = {k: torch.as_tensor(v).to(dev) for k, v in flat.items()}
        d = self._dev
        self._c = _lib.Basis(basis.molecule.natom(), basis.nshell(), basis.ncart(),
                             int(max(sh.l for sh in basis.shells)),
                             *(d[k].data_ptr() for k in
                               ("atom_xyz", "atom_charge", "shell_l", "shell_atom", "shell_nprim", "shell_prim0",
                                "shell_cart0", "bf_shell", "exps", "coefs")))
        self._rows = None
        if basis.pure and any(sh.l >= 1 for sh in basis.shells):
            T = basis.cart_to_ao()
            nbf = basis.nbf()
            cart0 = np.zeros(nbf, dtype=np.int32)
            length = np.zeros(nbf, dtype=np.int32)
            coef = np.zeros((nbf, _lib.AO_ROW_MAX))
            for sh in basis.shells:
                nr = 2 * sh.l + 1
                for r in range(nr):
                    row = T[sh.bf0 + r, sh.cart0:sh.cart0 + sh.ncart]
                    cart0[sh.bf0 + r] = sh.cart0
                    length[sh.bf0 + r] = sh.ncart
                    coef[sh.bf0 + r, :sh.ncart] = row
            self._rows = tuple(torch.as_tensor(a).to(dev) for a in (cart0, length, coef))

    # ------------------------------------------------------------------ kernels
    def _to_ao(self, x, ndim_ao):
        """Apply the Cartesian -> pure transform to the last ``ndim_ao`` axes."""
        if self._rows is None:
            return x
        nc, nbf = self.basis.ncart(), self.basis.nbf()
        cart0, length, coef = self._rows
        shape = list(x.shape)
        for ax in range(x.dim() - ndim_ao, x.dim()):
            pre = int(np.prod(shape[:ax])) if ax > 0 else 1
            post = int(np.prod(shape[ax + 1:])) if ax + 1 < len(shape) else 1
            shape[ax] = nbf
            out = torch.empty(shape, dtype=torch.float64, device=x.device)
            _lib.call("agb_ao_transform_axis", ptr(x), pre, nc, post, nbf, ptr(cart0), ptr(length), ptr(coef),
                      ptr(out), stream_ptr())
            x = out
        return x

    def _oei(self, kind, origin=None):
        nc = self.basis.ncart()
        ncomp = 3 if kind >= _lib.OEI_DIPOLE else 1
        out = torch.empty((ncomp, nc, nc), dtype=torch.float64, device=device())
        org = (ctypes.c_double * 3)(*(origin if origin is not None else (0.0, 0.0, 0.0)))
        _lib.call("agb_ao_one_electron", ctypes.byref(self._c), kind, org, ptr(out), stream_ptr())
        return self._to_ao(out, 2)

    def _single(self, kind, return_torch):
        m = self._oei(kind)[0]
        return m if return_torch else _host(m)

    def _triple(self, kind, origin, return_torch):
        m = self._oei(kind, origin)
        return [m[k] for k in range(3)] if return_torch else [_host(m[k]) for k in range(3)]

    # ------------------------------------------------------------------ psi4 names
    def ao_overlap(self, bs1=None, bs2=None, return_torch=False):
        """<bs1|bs2> (psi4's two-basis form); the basis of this helper when omitted."""
        if bs1 is None and bs2 is None:
            return self._single(_lib.OEI_OVERLAP, return_torch)
        bs1 = self.basis if bs1 is None else bs1
        bs2 = self.basis if bs2 is None else bs2
        n1 = bs1.nbf()
        m = MintsHelper(bs1.union(bs2))._oei(_lib.OEI_OVERLAP)[0][:n1, n1:].contiguous()
        return m if return_torch else _host(m)

    def ao_kinetic(self, return_torch=False):
        return self._single(_lib.OEI_KINETIC, return_torch)

    def ao_potential(self, return_torch=False):
        return self._single(_lib.OEI_POTENTIAL, return_torch)

    def ao_dipole(self, origin=None, return_torch=False):
        return self._triple(_lib.OEI_DIPOLE, origin, return_torch)

    def ao_nabla(self, return_torch=False):
        return self._triple(_lib.OEI_NABLA, None, return_torch)

    def ao_angular_momentum(self, origin=None, return_torch=False):
        return self._triple(_lib.OEI_ANGMOM, origin, return_torch)

    # ------------------------------------------------------------------ nuclear derivatives
    def oei_deriv_all(self, kind):
        """[natom, 3, nbf, nbf] device tensor of d(integral)/dR for OVERLAP, KINETIC,
        POTENTIAL or OVERLAP_HALF (bra derivative only); [natom, 3, 3, nbf, nbf] for DIPOLE."""
        nc, na = self.basis.ncart(), self.basis.molecule.natom()
        shape = (na, 3, 3, nc, nc) if kind == _lib.OEI_DIPOLE else (na, 3, nc, nc)
        out = torch.empty(shape, dtype=torch.float64, device=device())
        _lib.call("agb_ao_one_electron_deriv", ctypes.byref(self._c), kind, ptr(out), stream_ptr())
        return self._to_ao(out, 2)

    def eri_deriv_all(self):
        """[natom, 3, nbf, nbf, nbf, nbf] device tensor of d(mn|ls)/dR."""
        nc, na = self.basis.ncart(), self.basis.molecule.natom()
        out = torch.empty((na, 3, nc, nc, nc, nc), dtype=torch.float64, device=device())
        _lib.call("agb_ao_eri_deriv", ctypes.byref(self._c), ptr(out), stream_ptr())
        return self._to_ao(out, 4)

    _KINDS = {"OVERLAP": _lib.OEI_OVERLAP, "KINETIC": _lib.OEI_KINETIC, "POTENTIAL": _lib.OEI_POTENTIAL}

    def ao_oei_deriv1(self, oei_type, atom, return_torch=False):
        """psi4's ao_oei_deriv1: [d/dx, d/dy, d/dz] of OVERLAP / KINETIC / POTENTIAL for one atom."""
        m = self.oei_deriv_all(self._KINDS[oei_type.upper()])[atom]
        return [m[c] for c in range(3)] if return_torch else [_host(m[c]) for c in range(3)]

    def ao_tei_deriv1(self, atom, return_torch=False):
        """psi4's ao_tei_deriv1: [d/dx, d/dy, d/dz] of the ERIs for one atom."""
        m = self.eri_deriv_all()[atom]
        return [m[c] for c in range(3)] if return_torch else [_host(m[c]) for c in range(3)]

    def ao_overlap_half_deriv1(self, side, atom, return_torch=False):
        """psi4's ao_overlap_half_deriv1: <d mu/dR | nu> ('LEFT') or <mu | d nu/dR> ('RIGHT')."""
        m = self.oei_deriv_all(_lib.OEI_OVERLAP_HALF)[atom]
        if side.upper() == "RIGHT":
            m = m.transpose(-1, -2).contiguous()
        return [m[c] for c in range(3)] if return_torch else [_host(m[c]) for c in range(3)]

    def ao_eri(self, return_torch=False):
        nc = self.basis.ncart()
        out = torch.empty((nc, nc, nc, nc), dtype=torch.float64, device=device())
        _lib.call("agb_ao_eri", ctypes.byref(self._c), ptr(out), stream_ptr())
        out = self._to_ao(out, 4)
        return out if return_torch else _host(out)
