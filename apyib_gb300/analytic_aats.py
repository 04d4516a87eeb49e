"""Analytic atomic axial tensors of RHF, MP2, CID and CISD wavefunctions at zero
field (the quantity of apyib/analytic_aats.py:30-1390), from one solve plus
first-order responses.

The AAT is I[R, B] = Im d^2 <Psi(R) | Psi(B)> / dR dB, the mixed second
derivative of the overlap between the wavefunction displaced along a nuclear
coordinate R and the one in a magnetic field B.  To first order in each
perturbation,

  * orbitals: phi(R) = chi(R) C (1 + R U^R), phi(B) = chi C (1 + B U^B), so the
    spin-orbital MO overlap is S(R, B) = 1 + R X + B Y + R B X Y with
    X = U^R^H + C^H <d chi/dR | chi> C (the half-derivative overlap) and Y = U^B;
  * amplitudes: t(R) = t + R t^R, t(B) = t + B t^B (normalised as the state is).

U^R (real) and U^B (imaginary) come from the closed-shell CPHF equations
(nuclear: gradient.py; magnetic: (e_a - e_i) X_ai + sum_bk [(ak|ib) - (ab|ik)] X_bk
= -Y_ai for U^B = i X, h^B = i Y = (i/2) L in the MO basis, U^B zero within the
occupied and within the virtual space), t^R and t^B from the amplitude response
(response.solve_responses, all perturbations in lockstep) with the derivative Hamiltonians in the MO basis
(skeleton integrals + U^H F + F U + G[dD], and the U terms of the ERIs).  The
overlap sums over reference, singly and doubly excited determinants are then the
Schur-complement contractions of aats.AAT applied to this exactly linearised
model; its mixed derivative is taken by a central difference over the model's
small parameter (1e-4), which needs no further solves: the model's pure-R and
pure-B parts cancel exactly, leaving an O(eps^2) remainder of ~1e-8 (measured
against the two-step Richardson value, ``steps=(1e-3, 5e-4)``, which agrees with
the reference's analytic goldens to 6e-8).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .aats import AAT
from .device import device, ptr, stream_ptr, to_dev, workspace
from .linalg import apply_axis, cg_solve, jk_fock, zmm


def _ao2mo(ERI_AO, C):
    """(pq|rs) = sum conj(C_mp) C_nq conj(C_lr) C_ss (mn|ls) for a real AO tensor (GPU)."""
    nbf = C.shape[0]
    out = torch.empty((nbf, nbf, nbf, nbf), dtype=torch.complex128, device=device())
    nb = _lib.load().agb_ao2mo_scratch_bytes(nbf, nbf, _lib.PREC_FP64)
    buf, sp, n = workspace(nb)
    _lib.call("agb_ao2mo", ptr(ERI_AO.contiguous()), nbf, ptr(C), nbf, ptr(out), sp, n, _lib.PREC_FP64,
              stream_ptr())
    return out


def _u_terms(G, U):
    """First-order change of (pq|rs) when C -> C (1 + U): one index at a time, each a
    library GEMM over the other three."""
    Uc = U.conj().resolve_conj()
    return apply_axis(G, Uc, 0) + apply_axis(G, U, 1) + apply_axis(G, Uc, 2) + apply_axis(G, U, 3)


def _mo(Cc, M):
    """C^H M C for an AO matrix M (library GEMMs)."""
    return zmm(zmm(Cc, M.to(torch.complex128), transA=True, conjA=True), Cc)


class analytic_derivative(object):
    """apyib/analytic_aats.py:14-29 interface: analytic_derivative(parameters)."""

    def __init__(self, parameters):
        from .gradient import _real_orbitals
        from .hamiltonian import Hamiltonian
        from .hf_wfn import hf_wfn
        if any(f != 0.0 for f in parameters["F_el"]) or any(f != 0.0 for f in parameters["F_mag"]):
            raise ValueError("analytic AATs are defined at zero field")
        self.parameters = parameters
        self.H = Hamiltonian(parameters)
        self.wfn = hf_wfn(self.H)
        E_scf, C = self.wfn.solve_SCF(parameters)
        self.C = _real_orbitals(C)
        self.wfn.C = self.C

    # ------------------------------------------------------------------ orbital responses
    def _setup(self):
        from .integrals import MintsHelper
        wfn, H = self.wfn, self.H
        nbf, no = wfn.nbf, wfn.ndocc
        nv = nbf - no
        self.nbf, self.no = nbf, no
        natom = H.molecule.natom()
        self.natom = natom
        eps = np.asarray(wfn.eps).real
        self.eps = eps
        C = to_dev(self.C, torch.float64)
        Cc = C.to(torch.complex128)
        self.Cc = Cc
        m = MintsHelper(H.basis_set)
        ERI_AO = to_dev(H.ERI, torch.float64)
        self.ERI_AO = ERI_AO
        G = _ao2mo(ERI_AO, Cc)                                    # all-MO (pq|rs)
        self.G = G
        Gr = G.real.to(torch.complex128)                          # real orbitals: real integrals
        o, v = slice(0, no), slice(no, nbf)
        dev = C.device
        e = torch.as_tensor(eps).to(dev)
        de = (e[no:, None] - e[None, :no]).reshape(-1)            # e_a - e_i, (a, i) row-major
        Co = Cc[:, :no].contiguous()
        Dh = zmm(Co, Co, transB=True, conjB=True)
        zero = torch.zeros((nbf, nbf), dtype=torch.complex128, device=dev)
        h_AO = to_dev(np.asarray(H.T) + np.asarray(H.V))
        F_AO = jk_fock(ERI_AO, Dh, h_AO, 1.0)
        self.F_MO = _mo(Cc, F_AO)
        # nuclear CPHF (real), U_oo = -S_oo / 2, U_vv = -S_vv / 2
        Sd = m.oei_deriv_all(_lib.OEI_OVERLAP)
        hd = m.oei_deriv_all(_lib.OEI_KINETIC) + m.oei_deriv_all(_lib.OEI_POTENTIAL)
        Hd = m.oei_deriv_all(_lib.OEI_OVERLAP_HALF)
        Gd = m.eri_deriv_all()
        A = (4.0 * Gr[v, o, v, o] - Gr[v, v, o, o].permute(0, 2, 1, 3) - Gr[v, o, o, v].permute(0, 2, 3, 1))
        A = A.reshape(nv * no, nv * no) + torch.diag(de.to(torch.complex128))
        Gvooo = (2.0 * Gr[v, o, o, o] - Gr[v, o, o, o].permute(0, 2, 1, 3)).reshape(nv * no, no * no)
        rhs, self.SR, self.skelF, self.skelG, self.HR = [], [], [], [], []
        for K in range(natom):
            for c in range(3):
                GR = Gd[K, c].contiguous()
                dF_AO = hd[K, c].to(torch.complex128) + jk_fock(GR, Dh, zero, 1.0)
                Fm = _mo(Cc, dF_AO)
                S = _mo(Cc, Sd[K, c])
                # B_ai = F^R_ai - S_ai e_i - sum_kl S_kl [2(ai|kl) - (ak|il)]
                B = Fm[v, o] - S[v, o] * e[None, :no] - zmm(Gvooo, S[o, o].reshape(-1, 1)).reshape(nv, no)
                rhs.append(-B.reshape(-1))
                self.SR.append(S)
                self.skelF.append(Fm)
                self.skelG.append(_ao2mo(GR, Cc))
                self.HR.append(_mo(Cc, Hd[K, c]))
        X = cg_solve(A, torch.stack(rhs, dim=1))
        nf = H.basis_set.n_frozen_core()
        self.nfzc = nf
        idx = torch.arange(no, device=dev)
        cross = (idx[:, None] < nf) != (idx[None, :] < nf)         # frozen-active pairs
        den = (e[None, :no] - e[:no, None]).to(torch.complex128)
        den = torch.where(cross, den, torch.ones_like(den))
        if nf:
            M1 = (4.0 * Gr[o, o, v, o] - Gr[o, v, o, o].permute(0, 2, 1, 3)
                  - Gr[o, o, o, v].permute(0, 2, 3, 1)).reshape(no * no, nv * no)
            M2 = (2.0 * Gr[o, o, o, o] - Gr[o, o, o, o].permute(0, 2, 1, 3)).reshape(no * no, no * no)
        self.UR = []
        for n, S in enumerate(self.SR):
            U = -0.5 * S.clone()
            U[v, o] = X[:, n].reshape(nv, no)
            U[o, v] = -S[o, v] - U[v, o].T
            if nf:
                # frozen-active rotations change a frozen-core energy: the orbitals stay canonical,
                # U_ij = (F^R_ij - e_j S_ij + G[dD]_ij) / (e_j - e_i) for i, j in different blocks
                Gdd = (zmm(M1, U[v, o].reshape(-1, 1)) - zmm(M2, S[o, o].reshape(-1, 1))).reshape(no, no)
                Bo = self.skelF[n][o, o] - S[o, o] * e[None, :no] + Gdd
                U[o, o] = torch.where(cross, Bo / den, U[o, o])
            self.UR.append(U.contiguous())
        # magnetic CPHF: U^B = i X with X_ai real, X_ia = X_ai, zero within occ and within vir
        L = m.ao_angular_momentum(return_torch=True)
        Am = (Gr[v, o, o, v].permute(0, 2, 3, 1) - Gr[v, v, o, o].permute(0, 2, 1, 3)).reshape(nv * no, nv * no)
        Am = Am + torch.diag(de.to(torch.complex128))
        self.hB, rhsB, Ys = [], [], []
        for b in range(3):
            Y = _mo(Cc, 0.5 * L[b])                              # h^B = i Y (MO), Y real
            Ys.append(Y)
            self.hB.append(1j * Y)
            rhsB.append(-Y[v, o].reshape(-1))
        self.Am = Am
        XB = cg_solve(Am, torch.stack(rhsB, dim=1))
        if nf:
            N1 = Gr[o, o, v, o].permute(0, 3, 2, 1).reshape(no * no, nv * no)     # (ik|bj) as [i, j, (b, k)]
            N2 = Gr[o, v, o, o].permute(0, 3, 1, 2).reshape(no * no, nv * no)     # (ib|kj) as [i, j, (b, k)]
        self.UB = []
        for b in range(3):
            U = torch.zeros((nbf, nbf), dtype=torch.complex128, device=dev)
            Xvo = XB[:, b].reshape(nv, no)
            U[v, o] = 1j * Xvo
            U[o, v] = 1j * Xvo.T
            if nf:
                # canonical frozen-active rotations: U_ij = (h^B_ij + G[dD]_ij) / (e_j - e_i),
                # G[dD]_ij = i sum_bk X_bk [(ik|bj) - (ib|kj)]
                Gdd = zmm(N1 - N2, Xvo.reshape(-1, 1)).reshape(no, no)
                U[o, o] = torch.where(cross, 1j * (Ys[b][o, o] + Gdd) / den, U[o, o])
            self.UB.append(U.contiguous())

    def _dH(self, U, skelF=None, skelG=None, hx=None):
        """MO derivative Fock matrix and ERIs for orbital response U (+ skeleton parts)."""
        Cc, no, nbf = self.Cc, self.no, self.nbf
        zero = torch.zeros((nbf, nbf), dtype=torch.complex128, device=Cc.device)
        dC = zmm(Cc, U)
        Co, dCo = Cc[:, :no].contiguous(), dC[:, :no].contiguous()
        dD = zmm(dCo, Co, transB=True, conjB=True) + zmm(Co, dCo, transB=True, conjB=True)
        dF = (zmm(U, self.F_MO, transA=True, conjA=True) + zmm(self.F_MO, U)
              + _mo(Cc, jk_fock(self.ERI_AO, dD.contiguous(), zero, 1.0)))
        if skelF is not None:
            dF = dF + skelF
        if hx is not None:
            dF = dF + hx
        dG = _u_terms(self.G, U)
        if skelG is not None:
            dG = dG + skelG
        return dF, dG

    # ------------------------------------------------------------------ amplitudes and responses
    def _amplitudes(self, singles, precision):
        from .cisd import CISDPlan, solve
        from .response import solve_responses
        from .utils import compute_F_SO
        no, nbf, nf = self.no, self.nbf, self.nfzc
        o, v = 2 * (no - nf), 2 * (nbf - no)
        eps = self.eps
        eps_so = np.concatenate([np.repeat(eps[nf:no], 2), np.repeat(eps[no:], 2)])
        P = dict(self.parameters)
        t_ = slice(nf, nbf)
        # 'mixed': the amplitudes by the mixed solve and the responses with FP64-accurate
        # tensor-core / double-float residual GEMMs instead of the FP64 pipe
        mixed = precision == "mixed"
        plan = CISDPlan(o, v, singles=singles, mixed=mixed)
        plan.set_fock(compute_F_SO(None, self.F_MO[t_, t_].contiguous(), return_torch=True), eps_so)
        plan.blocks_from_mo(self.G[t_, t_, t_, t_].contiguous())
        E, t = solve(plan, P, precision=precision)

        def perturbed_plan(dF, dG):
            px = CISDPlan(o, v, singles=singles, mixed=mixed)
            px.set_fock(compute_F_SO(None, dF[t_, t_].contiguous(), return_torch=True), eps_so)
            px.blocks_from_mo(dG[t_, t_, t_, t_].contiguous())
            return px
        pert = [(self.UR[n], dict(skelF=self.skelF[n], skelG=self.skelG[n])) for n in range(len(self.UR))]
        pert += [(self.UB[b], dict(hx=self.hB[b])) for b in range(3)]
        # the 3N + 3 responses solved in lockstep, in batches whose plans and DIIS histories
        # (~25 amplitude vectors each) stay within a quarter of the free device memory
        per = plan._ws_buf.numel() + 25 * 16 * (plan.n1 + plan.n2)
        batch = int(max(1, min(len(pert), torch.cuda.mem_get_info()[0] // 4 // per)))
        tx = []
        for b0 in range(0, len(pert), batch):
            pxs = [perturbed_plan(*self._dH(U, **kw)) for U, kw in pert[b0:b0 + batch]]
            tx += [x for _, x in solve_responses(plan, pxs, t, E, P, precision="ozaki" if mixed else "fp64")]
            del pxs
        unpack = plan.unpack
        n3 = len(self.UR)
        return unpack(t), [unpack(x) for x in tx[:n3]], [unpack(x) for x in tx[n3:]]

    def _mp2_amplitudes(self):
        """MP2 first-order amplitudes t = <ab||ij> / (e_i + e_j - e_a - e_b) (apyib/mp2_wfn.py:
        64-87) and their responses from the first-order non-canonical MP2 equation
        <ab||ij> + P(F_vv t) - P(F_oo t) = 0 (the Fock terms of apyib/ci_wfn.py:324-327):
        t^x = [<ab||ij>^x + F^x_bc t_ijac + F^x_ac t_ijcb - F^x_kj t_ikab - F^x_ki t_kjab] / D."""
        from .adjoint import mp2_fock_apply
        from .utils import compute_ERI_SO, compute_F_SO
        no, nbf, nf = self.no, self.nbf, self.nfzc
        o = 2 * (no - nf)
        t_ = slice(nf, nbf)
        e = torch.as_tensor(np.repeat(self.eps[nf:], 2)).to(self.Cc.device)
        D = e[:o, None, None, None] + e[None, :o, None, None] - e[None, None, o:, None] - e[None, None, None, o:]

        def antisym(Gmo):
            Gs = compute_ERI_SO(None, Gmo[t_, t_, t_, t_].contiguous(), return_torch=True)[o:, :o, o:, :o]  # (a i|b j)
            return Gs.permute(1, 3, 0, 2) - Gs.permute(3, 1, 0, 2)                # <ab||ij> as [i,j,a,b]
        t = antisym(self.G) / D

        def respond(dF, dG):
            Fs = compute_F_SO(None, dF[t_, t_].contiguous(), return_torch=True)
            Fo, Fv = Fs[:o, :o], Fs[o:, o:]
            r = antisym(dG) + mp2_fock_apply(t, Fo, Fv)
            return (None, r / D)
        tR = [respond(*self._dH(self.UR[n], self.skelF[n], self.skelG[n])) for n in range(len(self.UR))]
        tB = [respond(*self._dH(self.UB[b], hx=self.hB[b])) for b in range(3)]
        return (None, t), tR, tB

    def _so(self, M):
        n = M.shape[0]
        S = torch.zeros((2 * n, 2 * n), dtype=torch.complex128, device=M.device)
        S[0::2, 0::2] = M
        S[1::2, 1::2] = M
        return S

    def _aats(self, method, normalization, precision="fp64", steps=(1e-4,), setup=True):
        """The AAT tensor; ``setup=False`` reuses the orbital responses already in place
        (the velocity-gauge APT replaces the magnetic ones)."""
        if setup:
            self._setup()
        nso = 2 * self.nbf
        eye = torch.eye(nso, dtype=torch.complex128, device=self.Cc.device)
        Xs = [self._so(U.conj().T + Hr) for U, Hr in zip(self.UR, self.HR)]
        Ys = [self._so(U) for U in self.UB]
        singles = method in ("CISD", "CISD_SO")
        if method == "RHF":
            T0, TR, TB = (None, None), [(None, None)] * len(Xs), [(None, None)] * 3
        elif method in ("MP2", "MP2_SO"):
            T0, TR, TB = self._mp2_amplitudes()
        else:
            T0, TR, TB = self._amplitudes(singles, precision)
        n3 = 3 * self.natom
        out = {}
        for eps in steps:
            ov = {"uu": eye}
            for b in range(3):
                ov["up", b], ov["un", b] = eye + eps * Ys[b], eye - eps * Ys[b]
            for a in range(n3):
                ov["pu", a], ov["nu", a] = eye + eps * Xs[a], eye - eps * Xs[a]
                for b in range(3):
                    XY = eps * eps * zmm(Xs[a], Ys[b])
                    ov["pp", a, b] = eye + eps * Xs[a] + eps * Ys[b] + XY
                    ov["pn", a, b] = eye + eps * Xs[a] - eps * Ys[b] - XY
                    ov["np", a, b] = eye - eps * Xs[a] + eps * Ys[b] - XY
                    ov["nn", a, b] = eye - eps * Xs[a] - eps * Ys[b] + XY

            def amp(base, d, s):
                if base[0] is None and base[1] is None and method == "RHF":
                    return [1.0, 0, 0]
                t1 = None if base[0] is None else base[0] + s * eps * d[0]
                t2 = base[1] + s * eps * d[1]
                return [1.0, t1, t2]
            so_method = method if method.endswith("_SO") or method == "RHF" else method + "_SO"
            A = AAT.from_overlaps({"method": so_method}, ndocc=self.no, nbf=self.nbf, nfzc=self.nfzc,
                                  natom=self.natom,
                                  overlaps=ov, unperturbed_T=amp(T0, (0, 0), 0),
                                  nuc_pos_T=[amp(T0, TR[a], 1) for a in range(n3)],
                                  nuc_neg_T=[amp(T0, TR[a], -1) for a in range(n3)],
                                  mag_pos_T=[amp(T0, TB[b], 1) for b in range(3)],
                                  mag_neg_T=[amp(T0, TB[b], -1) for b in range(3)],
                                  nuc_pert_strength=eps, mag_pert_strength=eps)
            out[eps] = A.compute_aat_tensor(normalization)
        if len(steps) == 1:
            return out[steps[0]]
        return (4 * out[steps[1]] - out[steps[0]]) / 3

    # ------------------------------------------------------------------ reference names
    def compute_RHF_AATs(self, orbitals="non-canonical"):
        return self._aats("RHF", "intermediate")

    def compute_MP2_AATs(self, normalization="full", orbitals="non-canonical"):
        return self._aats("MP2", normalization)

    def compute_CID_AATs(self, normalization="full", orbitals="non-canonical", print_level=0, precision="fp64"):
        """precision 'fp64' (the reference's arithmetic) or 'mixed' (FP64-accurate
        residual GEMMs off the FP64 pipe for the amplitudes and their responses)."""
        return self._aats("CID", normalization, precision=precision)

    def compute_CISD_AATs(self, normalization="full", orbitals="non-canonical", print_level=0, precision="fp64"):
        """precision as compute_CID_AATs."""
        return self._aats("CISD", normalization, precision=precision)
