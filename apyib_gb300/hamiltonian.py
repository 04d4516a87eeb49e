"""The Hamiltonian object the hot path consumes (interface of apyib/hamiltonian.py:13-70).

The hot path reads ``T, V, S, ERI, E_nuc``, ``basis_set.nbf()``,
``basis_set.n_frozen_core()`` and ``molecule.natom()/true_atomic_number()``.
``Hamiltonian(parameters)`` builds the molecule and basis from
``parameters['geom']`` / ``['basis']`` (``apyib_gb300.basis``) and computes the
AO integrals on the GPU (``apyib_gb300.integrals.MintsHelper``): kinetic,
potential, ERI, overlap, and for non-zero fields the electric dipole and
magnetic terms V -= F_el.mu_el + F_mag.(-i/2 L), E_nuc with the field term, as
apyib/hamiltonian.py:29-70 does with psi4.  ``parameters['integrals'] = 'psi4'``
takes the integrals from psi4 instead, where it is installed.
``Hamiltonian.from_arrays`` builds the object from arrays.  The phase-space
Hamiltonians of apyib/hamiltonian.py:72-538 are not part of this hot path.
"""
from __future__ import annotations

import types

import numpy as np


class Hamiltonian(object):
    def __init__(self, parameters):
        if parameters.get("integrals", "native") != "psi4":
            return self._native(parameters)
        try:
            import psi4
        except ImportError as exc:  # pragma: no cover - depends on the environment
            raise ImportError("Hamiltonian(parameters) needs psi4 for AO integrals; "
                              "use Hamiltonian.from_arrays(...) without it") from exc
        psi4.core.clean_options()
        psi4.set_options({"basis": parameters["basis"]})
        psi4.set_options({"freeze_core": parameters["freeze_core"]})
        self.molecule = psi4.geometry(parameters["geom"])
        self.basis_set = psi4.core.BasisSet.build(self.molecule)
        mints = psi4.core.MintsHelper(self.basis_set)
        self.T = mints.ao_kinetic().np
        self.V = mints.ao_potential().np
        self.ERI = mints.ao_eri().np
        self.S = mints.ao_overlap().np
        E_field = any(parameters["F_el"][a] != 0.0 for a in range(3))
        M_field = any(parameters["F_mag"][a] != 0.0 for a in range(3))
        if E_field:
            self.mu_el = [m.np for m in mints.ao_dipole()]
        if M_field:
            self.mu_mag = [-0.5j * m.np for m in mints.ao_angular_momentum()]
        F_el = [-parameters["F_el"][a] for a in range(3)]
        self.E_nuc = self.molecule.nuclear_repulsion_energy(F_el)
        for a in range(3):
            if E_field:
                self.V = self.V - parameters["F_el"][a] * self.mu_el[a]
            if M_field:
                self.V = self.V - parameters["F_mag"][a] * self.mu_mag[a]

    def _native(self, parameters):
        from . import basis as _basis
        from .integrals import MintsHelper
        self.molecule = _basis.parse_geometry(parameters["geom"])
        self.basis_set = _basis.BasisSet.build(self.molecule, parameters["basis"], puream=parameters.get("puream"),
                                               freeze_core=bool(parameters["freeze_core"]))
        mints = MintsHelper(self.basis_set)
        self.T = mints.ao_kinetic().np
        self.V = mints.ao_potential().np
        self.ERI = mints.ao_eri().np
        self.S = mints.ao_overlap().np
        E_field = any(parameters["F_el"][a] != 0.0 for a in range(3))
        M_field = any(parameters["F_mag"][a] != 0.0 for a in range(3))
        if E_field:
            self.mu_el = [m.np for m in mints.ao_dipole()]
        if M_field:
            self.mu_mag = [-0.5j * m.np for m in mints.ao_angular_momentum()]
        F_el = [-parameters["F_el"][a] for a in range(3)]
        self.E_nuc = self.molecule.nuclear_repulsion_energy(F_el)
        for a in range(3):
            if E_field:
                self.V = self.V - parameters["F_el"][a] * self.mu_el[a]
            if M_field:
                self.V = self.V - parameters["F_mag"][a] * self.mu_mag[a]

    @classmethod
    def from_arrays(cls, T, V, S, ERI, E_nuc=0.0, nelec=None, nfzc=0):
        """A Hamiltonian from AO arrays: T, V (may be complex), S, real chemist ERI."""
        self = cls.__new__(cls)
        nbf = S.shape[0]
        self.T, self.V, self.S, self.ERI = np.asarray(T), np.asarray(V), np.asarray(S), np.asarray(ERI)
        self.E_nuc = E_nuc
        self.basis_set = types.SimpleNamespace(nbf=lambda: nbf, n_frozen_core=lambda: nfzc)
        self.molecule = types.SimpleNamespace(natom=lambda: 1, true_atomic_number=lambda a: nelec)
        return self
