"""Finite-difference atomic axial tensors from wavefunction overlaps
(apyib/aats.py:19-1067), with the determinant sums turned into contractions.

The reference evaluates every term <Phi_bra | Phi_ket> between reference,
singly and doubly excited determinants of two wavefunctions as the
determinant of the occupied block of their spin-orbital MO overlap S with rows
and columns swapped (apyib/aats.py:120-131), one determinant per excitation
pair: O(o^4 v^4) determinants for the doubles/doubles term.  Here, with
A = S_oo, B = S_vo A^-1, C = A^-1 S_ov and G = S_vv - S_vo A^-1 S_ov (the Schur
complement), the matrix determinant lemma gives for bra rows i_r -> a_r and
ket columns k_s -> c_s

    det S[bra, ket] = det(A) det | B[a_r, i_r']   -G[a_r, c_s'] |
                                 | A^-1[k_s, i_r']  C[k_s, c_s'] |

(at most 4x4), and summing it against antisymmetric amplitudes leaves a few
GEMM-shaped contractions per term, O(o^2 v^2 (o + v)) in all.  With weights
1 (singles) and 1/4 (doubles) per side, X1 = x.B, Y1 = y.C,
X2 = x_ijab B_ai B_bj, Y2 = y_klcd C_kc C_ld, Yc_kc = y_klcd C_ld,
Xb_jb = x_ijab B_ai and F(u) = A^-T u G^T:

    00: 1         01: Y1        02: Y2/2       10: X1        20: X2/2
    11: X1 Y1 + x.F(y)          12: X1 Y2/2 + x.F(Yc)
    21: Xb.F(y) + X2 Y1/2       22: X2 Y2/4 + Xb.F(Yc) + (x.(A^-T A^-T G G) y)/4

all times det(A).  The terms I_00 ... I_DS and their sum are then assembled
exactly as apyib/aats.py:161-555 does, with the same normalisations
(apyib/aats.py:134-158) and the same prefactor Im(I) / (4 h_R h_B).  MO
overlaps between geometries/fields come from the GPU integral source
(utils.compute_mo_overlap); det(A) and A^-1 (occupied x occupied) come from the
library's batched Gauss-Jordan kernel (agb_zdet_inv_batched) and every product and
sum from its batched complex GEMM (agb_zgemm_batched), all overlaps of a tensor at
once, in FP64.

Spatial-orbital AATs (apyib/aats.py:646-1067) are the same quantity: the
closed-shell amplitudes are expanded to spin orbitals (alpha even, beta odd)
and the spin-orbital terms evaluated.  Frozen core: excitations run over the
active occupied orbitals; the determinants include the frozen ones.
"""
from __future__ import annotations

import numpy as np
import torch

from .device import device, to_dev
from .linalg import bdet_inv, bdot, bmm
from .utils import compute_mo_overlap, compute_so_overlap


# ----------------------------------------------------------------------------- amplitudes
def so_amplitudes(t1, t2, spatial):
    """Spin-orbital (t1, t2) device tensors; spatial closed-shell amplitudes
    t2[i,j,a,b] = t_{i alpha j beta}^{a alpha b beta} are expanded."""
    t2 = None if t2 is None or np.isscalar(t2) else to_dev(t2)
    t1 = None if t1 is None or np.isscalar(t1) else to_dev(t1)
    if not spatial:
        return t1, t2
    o, _, v, _ = t2.shape
    T2 = torch.zeros((2 * o, 2 * o, 2 * v, 2 * v), dtype=torch.complex128, device=device())
    tba = t2.transpose(2, 3)                  # t[i,j,b,a]
    T2[0::2, 1::2, 0::2, 1::2] = t2
    T2[1::2, 0::2, 1::2, 0::2] = t2
    T2[0::2, 1::2, 1::2, 0::2] = -tba
    T2[1::2, 0::2, 0::2, 1::2] = -tba
    T2[0::2, 0::2, 0::2, 0::2] = t2 - tba
    T2[1::2, 1::2, 1::2, 1::2] = t2 - tba
    T1 = None
    if t1 is not None:
        T1 = torch.zeros((2 * o, 2 * v), dtype=torch.complex128, device=device())
        T1[0::2, 0::2] = t1
        T1[1::2, 1::2] = t1
    return T1, T2


class _Stack:
    """det(A), A^-1, B, C, G of a list of spin-orbital overlaps, stacked along a leading
    axis F and restricted to the active occupied orbitals [f, o) for the excitation
    indices, so that the terms of many overlaps run as one set of batched products on
    the library (agb_zdet_inv_batched for det(A) and A^-1, agb_zgemm_batched for every
    product and sum).  Amplitudes passed to q_all carry a leading axis of length F or 1
    (shared)."""

    def __init__(self, Ss, o, f):
        S = torch.stack([to_dev(x) for x in Ss])
        self.det, Ai = bdet_inv(S[:, :o, :o])                                  # [F], [F, o, o]
        SOV, SVO = S[:, :o, o:], S[:, o:, :o]
        C = bmm(Ai, SOV)                                                        # [F, o, v]
        B = bmm(SVO, Ai)                                                        # [F, v, o]
        self.G = S[:, o:, o:] - bmm(SVO, C)                                     # [F, v, v]
        self.BT = B[:, :, f:].transpose(1, 2).contiguous()                      # [F, o_act, v]
        self.C = C[:, f:, :].contiguous()                                       # [F, o_act, v]
        self.Ai = Ai[:, f:, f:].contiguous()                                    # A^-1 on the active indices

    def F(self, u):
        """A^-T u G^T, u [F or 1, o_act, v]."""
        return bmm(bmm(self.Ai, u, transA=True), self.G, transB=True)

    def q_all(self, pairs, x, y):
        """{(r, s): det * <bra rank r (amplitudes x[r]) | ket rank s (y[s])>} for the
        requested rank pairs, each a tensor [F]; x, y: {rank: stacked amplitudes}."""
        need_r = {r for r, _ in pairs}
        need_s = {s for _, s in pairs}
        X1 = X2 = Xb = Y1 = Y2 = Yc = None
        if 1 in need_r:
            X1 = bdot(x[1], self.BT)
        if 2 in need_r:
            x2 = x[2]
            Fx, no, _, nv, _ = x2.shape
            xm = x2.permute(0, 1, 3, 2, 4).reshape(Fx, no * nv, no * nv)            # [(i,a),(j,b)]
            Xb = bmm(self.BT.reshape(self.BT.shape[0], 1, no * nv), xm).reshape(-1, no, nv)   # sum_ia x_ijab B_ai
            X2 = bdot(Xb, self.BT)
        if 1 in need_s:
            Y1 = bdot(y[1], self.C)
        if 2 in need_s:
            y2 = y[2]
            Fy, no, _, nv, _ = y2.shape
            ym = y2.permute(0, 2, 4, 1, 3).reshape(Fy, no * nv, no * nv)            # [(l,d),(k,c)]
            Yc = bmm(self.C.reshape(self.C.shape[0], 1, no * nv), ym).reshape(-1, no, nv)     # sum_ld y_klcd C_ld
            Y2 = bdot(Yc, self.C)
        out = {}
        for r, s in pairs:
            if r == 0 and s == 0:
                val = torch.ones_like(self.det)
            elif r == 0:
                val = Y1 if s == 1 else 0.5 * Y2
            elif s == 0:
                val = X1 if r == 1 else 0.5 * X2
            elif r == 1 and s == 1:
                val = X1 * Y1 + bdot(x[1], self.F(y[1]))
            elif r == 1 and s == 2:
                val = 0.5 * X1 * Y2 + bdot(x[1], self.F(Yc))
            elif r == 2 and s == 1:
                val = bdot(Xb, self.F(y[1])) + 0.5 * X2 * Y1
            else:
                # x.(A^-T A^-T G G) y = sum_klab (A^-1 A^-1 x)_klab (G G y)_klab: occupied
                # factors on x, virtual factors on y
                x2, y2 = x[2], y[2]
                no, nv = x2.shape[1], x2.shape[3]
                xa = bmm(self.Ai, x2.reshape(x2.shape[0], no, -1)).reshape(-1, no, no, nv, nv)      # k <- i
                xa = bmm(self.Ai, xa.transpose(1, 2).reshape(xa.shape[0], no, -1)).reshape(-1, no, no, nv, nv)
                xa = xa.transpose(1, 2)                                                          # [k, l, a, b]
                ya = bmm(y2.reshape(y2.shape[0], -1, nv), self.G, transB=True)                   # d <- b
                ya = ya.reshape(ya.shape[0], no * no, nv, nv).permute(0, 2, 1, 3).reshape(ya.shape[0], nv, -1)
                ya = bmm(self.G, ya)
                ya = ya.reshape(ya.shape[0], nv, no * no, nv).permute(0, 2, 1, 3)                # c <- a
                val = 0.25 * X2 * Y2 + bdot(Xb, self.F(Yc)) + 0.25 * bdot(xa, ya)
            out[r, s] = self.det * val
        return out


class _Factors:
    """_Stack of one overlap: q(r, x, s, y) is the single term as a device scalar."""

    def __init__(self, S, o, f):
        self._st = _Stack([S], o, f)
        self.det = self._st.det[0]

    def q(self, r, x, s, y):
        xs = {r: x.unsqueeze(0)} if r else {}
        ys = {s: y.unsqueeze(0)} if s else {}
        return self._st.q_all([(r, s)], xs, ys)[r, s][0]      # a device scalar: no host round trip per term


class AAT(object):
    """apyib/aats.py:19-118 with the same arguments; overlaps on the GPU."""

    def __init__(self, parameters, wfn, unperturbed_wfn, unperturbed_basis, unperturbed_T, nuc_pos_wfn, nuc_neg_wfn,
                 nuc_pos_basis, nuc_neg_basis, nuc_pos_T, nuc_neg_T, mag_pos_wfn, mag_neg_wfn, mag_pos_basis,
                 mag_neg_basis, mag_pos_T, mag_neg_T, nuc_pert_strength, mag_pert_strength):
        self.parameters = parameters
        self.nbf = wfn.nbf
        self.ndocc = wfn.ndocc
        self.nfzc = wfn.H.basis_set.n_frozen_core()
        self.natom = wfn.H.molecule.natom()
        nbf, no = self.nbf, self.ndocc

        def so(bra_b, bra_c, ket_b, ket_c):
            return compute_so_overlap(nbf, compute_mo_overlap(no, nbf, bra_b, bra_c, ket_b, ket_c, return_torch=True),
                                      return_torch=True)
        ub, uc = unperturbed_basis, unperturbed_wfn
        n3 = 3 * self.natom
        ov = {}
        correlated = parameters["method"] != "RHF"
        if correlated:
            ov["uu"] = so(ub, uc, ub, uc)
            for b in range(3):
                ov["up", b] = so(ub, uc, mag_pos_basis[b], mag_pos_wfn[b])
                ov["un", b] = so(ub, uc, mag_neg_basis[b], mag_neg_wfn[b])
            for a in range(n3):
                ov["pu", a] = so(nuc_pos_basis[a], nuc_pos_wfn[a], ub, uc)
                ov["nu", a] = so(nuc_neg_basis[a], nuc_neg_wfn[a], ub, uc)
        for a in range(n3):
            for b in range(3):
                ov["pp", a, b] = so(nuc_pos_basis[a], nuc_pos_wfn[a], mag_pos_basis[b], mag_pos_wfn[b])
                ov["pn", a, b] = so(nuc_pos_basis[a], nuc_pos_wfn[a], mag_neg_basis[b], mag_neg_wfn[b])
                ov["np", a, b] = so(nuc_neg_basis[a], nuc_neg_wfn[a], mag_pos_basis[b], mag_pos_wfn[b])
                ov["nn", a, b] = so(nuc_neg_basis[a], nuc_neg_wfn[a], mag_neg_basis[b], mag_neg_wfn[b])
        self._init_common(ov, unperturbed_T, nuc_pos_T, nuc_neg_T, mag_pos_T, mag_neg_T, nuc_pert_strength,
                          mag_pert_strength)

    @classmethod
    def from_overlaps(cls, parameters, ndocc, nbf, nfzc, natom, overlaps, unperturbed_T, nuc_pos_T, nuc_neg_T,
                      mag_pos_T, mag_neg_T, nuc_pert_strength, mag_pert_strength):
        """Build from spin-orbital overlap matrices keyed 'uu', ('up', b), ('un', b),
        ('pu', a), ('nu', a), ('pp', a, b), ('pn', a, b), ('np', a, b), ('nn', a, b)."""
        self = cls.__new__(cls)
        self.parameters = parameters
        self.ndocc, self.nbf, self.nfzc, self.natom = ndocc, nbf, nfzc, natom
        self._init_common(overlaps, unperturbed_T, nuc_pos_T, nuc_neg_T, mag_pos_T, mag_neg_T, nuc_pert_strength,
                          mag_pert_strength)
        return self

    def _init_common(self, ov, uT, npT, nnT, mpT, mnT, h, b):
        self._ov = ov
        self.nuc_pert_strength, self.mag_pert_strength = h, b
        method = self.parameters["method"]
        self.spatial = method in ("MP2", "CID", "CISD")
        self.singles = method in ("CISD", "CISD_SO")
        self.doubles = method != "RHF"

        def amps(T):
            if not self.doubles:
                return (1.0, None, None)
            t1, t2 = so_amplitudes(T[1] if self.singles else None, T[2], self.spatial)
            return (complex(T[0]), t1, t2)
        self.uT = amps(uT)
        self.npT = [amps(T) for T in npT] if self.doubles else None
        self.nnT = [amps(T) for T in nnT] if self.doubles else None
        self.mpT = [amps(T) for T in mpT] if self.doubles else None
        self.mnT = [amps(T) for T in mnT] if self.doubles else None

    @property
    def _f(self):
        """Per-overlap factors for the element-by-element terms (built on first use)."""
        if "_factors" not in self.__dict__:
            o, f = 2 * self.ndocc, 2 * self.nfzc
            self._factors = {k: _Factors(S, o, f) for k, S in self._ov.items()}
        return self._factors

    # ------------------------------------------------------------------ normalisation
    def _norm(self, T):
        key = id(T)
        cache = self.__dict__.setdefault("_norm_cache", {})
        if key not in cache:
            cache[key] = (T, self._norm_value(T))         # T kept alive so that its id stays unique
        return cache[key][1]

    def _norm_value(self, T):
        t0, t1, t2 = T
        s = t0 ** 2
        if t2 is not None:
            s = s + 0.25 * complex(torch.sum(t2.conj() * t2).item())
        if self.singles and t1 is not None:
            s = s + complex(torch.sum(t1.conj() * t1).item())
        return 1 / np.sqrt(s)

    def compute_normalization(self, alpha, beta, normalization):
        """apyib/aats.py:134-158 (and :653-672 for spatial amplitudes)."""
        if self.parameters["method"] == "RHF" or normalization == "intermediate":
            return 1, 1, 1, 1, 1
        return (self._norm(self.uT), self._norm(self.npT[alpha]), self._norm(self.nnT[alpha]),
                self._norm(self.mpT[beta]), self._norm(self.mnT[beta]))

    # ------------------------------------------------------------------ terms
    def _pref(self):
        return 1 / (4 * self.nuc_pert_strength * self.mag_pert_strength)

    def _four(self, alpha, beta, r, x, s, y, N):
        """x, y against the pp, pn, np, nn overlaps with their normalisations."""
        _, N_np, N_nn, N_mp, N_mn = N
        f = self._f
        return (f["pp", alpha, beta].q(r, x, s, y) * N_np * N_mp - f["pn", alpha, beta].q(r, x, s, y) * N_np * N_mn
                - f["np", alpha, beta].q(r, x, s, y) * N_nn * N_mp + f["nn", alpha, beta].q(r, x, s, y) * N_nn * N_mn)

    def _amp(self, alpha, beta, rank):
        """(t, t*, dt/dH, dt/dR*) of the given excitation rank (1 or 2)."""
        k = rank
        t = self.uT[k]
        return (t, t.conj(), self.mpT[beta][k] - self.mnT[beta][k], (self.npT[alpha][k] - self.nnT[alpha][k]).conj())

    def _term(self, alpha, beta, r, s, normalization):
        N = self.compute_normalization(alpha, beta, normalization)
        Nu, N_np, N_nn, N_mp, N_mn = N
        f = self._f
        if r == 0 and s == 0:
            I = self._four(alpha, beta, 0, None, 0, None, N)
            return self._pref() * I.imag
        I = 0
        if r == 0:
            t, _, tdH, _ = self._amp(alpha, beta, s)
            I += f["pu", alpha].q(0, None, s, tdH) * N_np * Nu - f["nu", alpha].q(0, None, s, tdH) * N_nn * Nu
            I += self._four(alpha, beta, 0, None, s, t, N)
        elif s == 0:
            _, tc, _, tdR = self._amp(alpha, beta, r)
            I += f["up", beta].q(r, tdR, 0, None) * Nu * N_mp - f["un", beta].q(r, tdR, 0, None) * Nu * N_mn
            I += self._four(alpha, beta, r, tc, 0, None, N)
        else:
            _, tc, _, tdR = self._amp(alpha, beta, r)
            t, _, tdH, _ = self._amp(alpha, beta, s)
            I += f["uu"].q(r, tdR, s, tdH) * Nu * Nu
            I += f["up", beta].q(r, tdR, s, t) * Nu * N_mp - f["un", beta].q(r, tdR, s, t) * Nu * N_mn
            I += f["pu", alpha].q(r, tc, s, tdH) * N_np * Nu - f["nu", alpha].q(r, tc, s, tdH) * N_nn * Nu
            I += self._four(alpha, beta, r, tc, s, t, N)
        return self._pref() * I.imag

    def _term_value(self, alpha, beta, r, s, normalization):
        return float(self._term(alpha, beta, r, s, normalization))

    def compute_SO_I_00(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 0, 0, normalization)

    def compute_SO_I_0D(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 0, 2, normalization)

    def compute_SO_I_D0(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 2, 0, normalization)

    def compute_SO_I_DD(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 2, 2, normalization)

    def compute_SO_I_0S(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 0, 1, normalization)

    def compute_SO_I_S0(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 1, 0, normalization)

    def compute_SO_I_SS(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 1, 1, normalization)

    def compute_SO_I_SD(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 1, 2, normalization)

    def compute_SO_I_DS(self, alpha, beta, normalization):
        return self._term_value(alpha, beta, 2, 1, normalization)

    def compute_SO_aats(self, alpha, beta, normalization="full"):
        """apyib/aats.py:520-555: the sum of the terms the method has."""
        terms = [(0, 0)]
        if self.doubles:
            terms += [(0, 2), (2, 0), (2, 2)]
        if self.singles:
            terms += [(0, 1), (1, 0), (1, 1), (1, 2), (2, 1)]
        return float(sum(self._term(alpha, beta, r, s, normalization) for r, s in terms))

    def compute_spatial_aats(self, alpha, beta, normalization="full"):
        """apyib/aats.py:646-1067: the same tensor from closed-shell amplitudes."""
        return self.compute_SO_aats(alpha, beta, normalization)

    def compute_aat_tensor(self, normalization="full"):
        """All 3N x 3 elements (the sum compute_SO_aats gives for each), every overlap
        term of every element evaluated at once: the overlaps are stacked and the
        contractions of the class docstring run as broadcast batched products."""
        n3 = 3 * self.natom
        o, f = 2 * self.ndocc, 2 * self.nfzc
        grid = [(a, b) for a in range(n3) for b in range(3)]
        pairs = [(0, 0)]
        if self.doubles:
            pairs += [(0, 2), (2, 0), (2, 2)]
        if self.singles:
            pairs += [(0, 1), (1, 0), (1, 1), (1, 2), (2, 1)]
        ranks = sorted(({r for r, _ in pairs} | {s for _, s in pairs}) - {0})

        def stack(keys):
            return _Stack([self._ov[k] for k in keys], o, f)

        def amps(get):
            """{rank: tensor stacked over the (a, b) grid}."""
            return {k: torch.stack([get(a, b, k) for a, b in grid]) for k in ranks}
        N = [self.compute_normalization(a, b, normalization) for a, b in grid]
        Nu = N[0][0]
        N_np, N_nn, N_mp, N_mn = (torch.as_tensor(np.array([complex(x[i]) for x in N])).to(device())
                                  for i in (1, 2, 3, 4))
        t = {k: self.uT[k][None] for k in ranks}
        tc = {k: self.uT[k].conj()[None] for k in ranks}
        # the four displaced/field overlaps of each element, unperturbed amplitudes on both sides
        q4 = [stack([(kind, a, b) for a, b in grid]).q_all(pairs, tc, t) for kind in ("pp", "pn", "np", "nn")]
        I = {}
        for r, s in pairs:
            I[r, s] = (q4[0][r, s] * N_np * N_mp - q4[1][r, s] * N_np * N_mn
                       - q4[2][r, s] * N_nn * N_mp + q4[3][r, s] * N_nn * N_mn)
        if self.doubles:
            tdH = amps(lambda a, b, k: self.mpT[b][k] - self.mnT[b][k])
            tdR = amps(lambda a, b, k: (self.npT[a][k] - self.nnT[a][k]).conj())
            pu, nu = stack([("pu", a) for a, b in grid]), stack([("nu", a) for a, b in grid])
            up, un = stack([("up", b) for a, b in grid]), stack([("un", b) for a, b in grid])
            ket = [(r, s) for r, s in pairs if r > 0 and s > 0]
            qpu = pu.q_all([(0, s) for s in ranks] + ket, tc, tdH)
            qnu = nu.q_all([(0, s) for s in ranks] + ket, tc, tdH)
            qup = up.q_all([(r, 0) for r in ranks], tdR, None)
            qun = un.q_all([(r, 0) for r in ranks], tdR, None)
            qup.update(up.q_all(ket, tdR, t))
            qun.update(un.q_all(ket, tdR, t))
            quu = stack(["uu"]).q_all(ket, tdR, tdH)
            for r, s in pairs:
                if r == 0 and s > 0:
                    I[r, s] = I[r, s] + (qpu[0, s] * N_np - qnu[0, s] * N_nn) * Nu
                elif s == 0 and r > 0:
                    I[r, s] = I[r, s] + (qup[r, 0] * N_mp - qun[r, 0] * N_mn) * Nu
                elif r > 0:
                    I[r, s] = (I[r, s] + quu[r, s] * Nu * Nu + (qup[r, s] * N_mp - qun[r, s] * N_mn) * Nu
                               + (qpu[r, s] * N_np - qnu[r, s] * N_nn) * Nu)
        total = sum(I[rs].imag for rs in pairs) / (4 * self.nuc_pert_strength * self.mag_pert_strength)
        return total.reshape(n3, 3).cpu().numpy()
