"""Finite-difference drivers (apyib/fin_diff.py:12-510) on the GPU energy path.

``finite_difference(parameters, unperturbed_basis, unperturbed_C)`` displaces
nuclei (and applies electric / magnetic fields) through ``parameters`` and runs
complete calculations (GPU integrals -> RHF -> the correlated method) at each
point:

* ``compute_Hessian(h)``: central differences of central-difference gradients,
  H[a, b] = (g_b(+h e_a) - g_b(-h e_a)) / 2h with
  g_b(x) = (E(x + h e_b) - E(x - h e_b)) / 2h (apyib/fin_diff.py:27-149);
* ``compute_APT(h, f)``: P[a, b] = (mu_b(+h e_a) - mu_b(-h e_a)) / 2h with
  mu_b = -(E(F_el,b = +f) - E(F_el,b = -f)) / 2f (apyib/fin_diff.py:151-265);
* ``compute_Nuclear_Gradient(h)``, ``compute_Magnetic_Field_Gradient(b)``:
  central differences of phase-corrected energies, with the displaced
  wavefunctions (apyib/fin_diff.py:376-510);
* ``compute_AAT(h, b)``: the phase-corrected wavefunctions at +-h on every
  nuclear coordinate and +-b on every magnetic-field component, the inputs of
  the overlap AATs (apyib/fin_diff.py:267-372).

The Hessian visits 4 (3N)^2 displaced geometries of which only about half are
distinct (E(x + h e_a + h e_b) = E(x + h e_b + h e_a)); energies are cached by
displacement, so each distinct geometry is solved once.  ``parameters`` is not
modified.
"""
from __future__ import annotations

import copy

import numpy as np

from .basis import parse_geometry
from .energy import energy, phase_corrected_energy


class finite_difference(object):
    def __init__(self, parameters, unperturbed_basis, unperturbed_C):
        self.parameters = parameters
        self.molecule = parse_geometry(parameters["geom"])
        self.geom = self.molecule.geometry()
        self.natom = self.molecule.natom()
        self.unperturbed_basis = unperturbed_basis
        self.unperturbed_C = unperturbed_C
        self._E = {}

    # ------------------------------------------------------------------ points
    def _point(self, disp=(), F_el=None, F_mag=None):
        """Parameters at geom + sum(mult * h e_coord) and the given field changes.
        disp: tuple of (coordinate, displacement in bohr)."""
        p = copy.deepcopy(self.parameters)
        if disp:
            g = self.geom.copy()
            for k, d in disp:
                g[k // 3][k % 3] += d
            mol = copy.deepcopy(self.molecule)
            mol.set_geometry(g)
            p["geom"] = mol.create_psi4_string_from_molecule()
        for key, delta in (("F_el", F_el), ("F_mag", F_mag)):
            if delta is not None:
                p[key] = [p[key][c] + delta[c] for c in range(3)]
        return p

    def _energy(self, key, params):
        if key not in self._E:
            E_list, _, _, _ = energy(params)
            self._E[key] = E_list[0] + E_list[1] + E_list[2]
        return self._E[key]

    def _nuc_energy(self, moves, h):
        """Total energy at geom + sum(m h e_k) for moves = {k: m}."""
        moves = {k: m for k, m in moves.items() if m != 0}
        key = ("nuc", h, tuple(sorted(moves.items())))
        return self._energy(key, self._point(tuple((k, m * h) for k, m in sorted(moves.items()))))

    # ------------------------------------------------------------------ drivers
    def compute_Hessian(self, nuc_pert_strength):
        h = nuc_pert_strength
        n = 3 * self.natom
        grad = {}
        for s in (1, -1):
            g = np.zeros((n, n), dtype=complex)
            for a in range(n):
                for b in range(n):
                    mp = {a: s}
                    mp[b] = mp.get(b, 0) + 1
                    mm = {a: s}
                    mm[b] = mm.get(b, 0) - 1
                    g[a, b] = (self._nuc_energy(mp, h) - self._nuc_energy(mm, h)) / (2 * h)
            grad[s] = g
        return (grad[1] - grad[-1]) / (2 * h)

    def compute_APT(self, nuc_pert_strength, elec_pert_strength):
        h, f = nuc_pert_strength, elec_pert_strength
        n = 3 * self.natom
        mu = {}
        for s in (1, -1):
            m = np.zeros((n, 3), dtype=complex)
            for a in range(n):
                for b in range(3):
                    e = []
                    for sf in (1, -1):
                        F = [0.0, 0.0, 0.0]
                        F[b] = sf * f
                        key = ("apt", h, a, s, f, b, sf)
                        e.append(self._energy(key, self._point(((a, s * h),), F_el=F)))
                    m[a, b] = -(e[0] - e[1]) / (2 * f)
            mu[s] = m
        return (mu[1] - mu[-1]) / (2 * h)

    def _wavefunctions(self, points):
        out = {"E": [], "C": [], "basis": [], "T": []}
        for p in points:
            E_list, T_list, C, basis = phase_corrected_energy(p, self.unperturbed_basis, self.unperturbed_C)
            out["E"].append(E_list[0] + E_list[1] + E_list[2])
            out["C"].append(C)
            out["T"].append(T_list)
            out["basis"].append(basis)
        return out

    def _nuc_points(self, h, sign):
        return [self._point(((a, sign * h),)) for a in range(3 * self.natom)]

    def _mag_points(self, b, sign):
        pts = []
        for beta in range(3):
            F = [0.0, 0.0, 0.0]
            F[beta] = sign * b
            pts.append(self._point(F_mag=F))
        return pts

    def compute_Nuclear_Gradient(self, nuc_pert_strength):
        h = nuc_pert_strength
        pos = self._wavefunctions(self._nuc_points(h, 1))
        neg = self._wavefunctions(self._nuc_points(h, -1))
        gradient = np.array([(pos["E"][k] - neg["E"][k]).real / (2 * h) for k in range(3 * self.natom)])
        return (gradient.reshape(self.natom, 3), pos["C"], neg["C"], pos["basis"], neg["basis"], pos["T"], neg["T"])

    def compute_Magnetic_Field_Gradient(self, mag_pert_strength):
        b = mag_pert_strength
        pos = self._wavefunctions(self._mag_points(b, 1))
        neg = self._wavefunctions(self._mag_points(b, -1))
        gradient = np.array([(pos["E"][k] - neg["E"][k]).real / (2 * b) for k in range(3)])
        return gradient, pos["C"], neg["C"], pos["basis"], neg["basis"], pos["T"], neg["T"]

    def compute_AAT(self, nuc_pert_strength, mag_pert_strength):
        npos = self._wavefunctions(self._nuc_points(nuc_pert_strength, 1))
        nneg = self._wavefunctions(self._nuc_points(nuc_pert_strength, -1))
        mpos = self._wavefunctions(self._mag_points(mag_pert_strength, 1))
        mneg = self._wavefunctions(self._mag_points(mag_pert_strength, -1))
        return (npos["C"], nneg["C"], npos["basis"], nneg["basis"], npos["T"], nneg["T"],
                mpos["C"], mneg["C"], mpos["basis"], mneg["basis"], mpos["T"], mneg["T"])
