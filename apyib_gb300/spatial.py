"""Closed-shell (spin-adapted) CISD / CID over complex spatial orbitals on the GPU
(apyib/ci_wfn.py:51-167 and :420-574).

The residual of the reference's spatial equations, term for term, with every
contraction one complex FP64 GEMM of the library (``linalg.zmm``) on reshaped
device tensors; the Jacobi update, the DIIS extrapolation of
apyib/utils.py:104-140 (history truncated to 7 before the append, iteration 1
not appended, bordered solve on the host in FP64) and the convergence test of
apyib/ci_wfn.py:520-535 (unconjugated squared norms, numpy's complex-versus-real
comparison) follow the reference.  Work per residual is that of the closed-shell
equations: about a sixteenth of the spin-orbital problem of the same molecule.

Amplitudes t1[i,a] (no x nv) and t2[i,j,a,b] (no, no, nv, nv); Dirac integrals
<pq|rs> = (pr|qs) from the chemist ERI_MO of the active space."""
from __future__ import annotations

import numpy as np
import torch

from .cisd import _bordered_diis, _lt
from .linalg import bdot, zmm


def _mm(A, B, transA=False, transB=False):
    return zmm(A.contiguous() if not A.is_contiguous() else A, B.contiguous() if not B.is_contiguous() else B,
               transA=transA, transB=transB)


class SpatialCISD:
    """The closed-shell residual and solver for one set of integrals (F_MO, ERI_MO on the
    device, complex128; ``no`` doubly occupied active orbitals first)."""

    def __init__(self, F_MO, ERI_MO, no, singles=True):
        n = F_MO.shape[0]
        self.no, self.nv, self.singles = no, n - no, singles
        o, v = slice(0, no), slice(no, n)
        g = ERI_MO.permute(0, 2, 1, 3)                                     # <pq|rs>
        self.F = F_MO
        self.Foo, self.Fvv, self.Fov = F_MO[o, o].contiguous(), F_MO[v, v].contiguous(), F_MO[o, v].contiguous()
        self.Fvo_T = F_MO[v, o].T.contiguous()                              # F_MO.swapaxes(0,1)[o,v]
        blk = lambda a, b, c, d: g[a, b, c, d].contiguous()
        self.g_oovv, self.g_vvoo = blk(o, o, v, v), blk(v, v, o, o)
        self.g_ovvo, self.g_ovov = blk(o, v, v, o), blk(o, v, o, v)
        self.g_oooo, self.g_vvvv = blk(o, o, o, o), blk(v, v, v, v)
        if singles:
            self.g_vovv, self.g_ooov, self.g_oovo = blk(v, o, v, v), blk(o, o, o, v), blk(o, o, v, o)
            self.g_vvvo, self.g_vvov = blk(v, v, v, o), blk(v, v, o, v)
            self.g_ovoo, self.g_vooo = blk(o, v, o, o), blk(v, o, o, o)
        # energy weights: E = 2 t1.F_ov + t2.(2 <ij|ab> - <ij|ba>) (apyib/ci_wfn.py:441,510)
        self.L_oovv = (2.0 * self.g_oovv - self.g_oovv.transpose(2, 3)).contiguous()
        eo = torch.diagonal(self.Foo).real
        ev = torch.diagonal(self.Fvv).real
        self.D_ia = (eo[:, None] - ev[None, :]).to(torch.complex128)
        self.D_ijab = (eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None]
                       - ev[None, None, None, :]).to(torch.complex128)

    def set_denominators(self, eps_o, eps_v):
        """Denominators from given orbital energies (the reference's wfn.eps slices)."""
        dev = self.F.device
        eo = torch.as_tensor(np.asarray(eps_o)).to(dev)
        ev = torch.as_tensor(np.asarray(eps_v)).to(dev)
        self.D_ia = (eo[:, None] - ev[None, :]).to(torch.complex128)
        self.D_ijab = (eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None]
                       - ev[None, None, None, :]).to(torch.complex128)

    # ------------------------------------------------------------------ residual
    def residual(self, t1, t2, E):
        """r_T1, r_T2 of apyib/ci_wfn.py:458-490 (CISD) or :84-111 (CID, t1 = None)."""
        no, nv = self.no, self.nv
        nov = no * nv
        r2 = self.g_vvoo.permute(2, 3, 0, 1).clone()                        # <ab|ij> as [i,j,a,b]
        r1 = None
        if self.singles:
            L_jbai = (2.0 * self.g_ovvo.permute(3, 1, 0, 2) - self.g_ovov.permute(2, 1, 0, 3)).reshape(nov, nov)
            t2x = (2.0 * t2 - t2.transpose(2, 3)).permute(0, 2, 1, 3).reshape(nov, nov)
            A_vovv = (2.0 * self.g_vovv - self.g_vovv.transpose(2, 3)).reshape(nv, no * nv * nv)
            B_ooov = (2.0 * self.g_ooov - self.g_oovo.permute(0, 1, 3, 2)).permute(2, 0, 1, 3).reshape(no, no * no * nv)
            r1 = self.Fvo_T.clone()
            r1 -= _mm(self.Foo, t1, transA=True)                                          # F_ji t1_ja
            r1 += _mm(t1, self.Fvv, transB=True)                                          # F_ab t1_ib
            r1 += _mm(L_jbai, t1.reshape(nov, 1)).reshape(no, nv)                         # (2<ja|bi> - <ja|ib>) t1_jb
            r1 += _mm(t2x, self.Fov.reshape(nov, 1)).reshape(no, nv)                      # F_jb (2 t2 - t2^T)
            r1 += _mm(t2.reshape(no, no * nv * nv), A_vovv, transB=True)                  # (2<aj|bc> - <aj|cb>) t2_ijbc
            r1 -= _mm(B_ooov, t2.permute(0, 1, 3, 2).reshape(no * no * nv, nv))           # (2<kj|ib> - <kj|bi>) t2_kjab
            r1 -= E * t1
            # t1 terms of the doubles
            X = _mm(t1, self.g_vvvo.permute(2, 0, 1, 3).reshape(nv, nv * nv * no))        # <ab|cj> t1_ic
            r2 += X.reshape(no, nv, nv, no).permute(0, 3, 1, 2)
            X = _mm(self.g_vvov.reshape(nv * nv * no, nv), t1, transB=True)               # <ab|ic> t1_jc
            r2 += X.reshape(nv, nv, no, no).permute(2, 3, 0, 1)
            X = _mm(t1, self.g_ovoo.reshape(no, nv * no * no), transA=True)               # <kb|ij> t1_ka
            r2 -= X.reshape(nv, nv, no, no).permute(2, 3, 0, 1)
            X = _mm(self.g_vooo.permute(0, 2, 3, 1).reshape(nv * no * no, no), t1)        # <ak|ij> t1_kb
            r2 -= X.reshape(nv, no, no, nv).permute(1, 2, 0, 3)
        T2 = t2.reshape(no * no * nv, nv)
        r2 += _mm(self.Fvv, t2.permute(2, 0, 1, 3).reshape(nv, -1)).reshape(nv, no, no, nv).permute(1, 2, 0, 3)
        r2 += _mm(T2, self.Fvv, transB=True).reshape(no, no, nv, nv)                    # F_bc t2_ijac
        r2 -= _mm(self.Foo, t2.reshape(no, -1), transA=True).reshape(no, no, nv, nv)    # F_ki t2_kjab
        r2 -= _mm(self.Foo, t2.permute(1, 0, 2, 3).reshape(no, -1), transA=True).reshape(no, no, nv, nv).permute(
            1, 0, 2, 3)                                                                  # F_kj t2_ikab
        r2 += _mm(self.g_oooo.reshape(no * no, no * no), t2.reshape(no * no, nv * nv), transA=True).reshape(
            no, no, nv, nv)                                                              # <kl|ij> t2_klab
        r2 += _mm(t2.reshape(no * no, nv * nv), self.g_vvvv.reshape(nv * nv, nv * nv), transB=True).reshape(
            no, no, nv, nv)                                                              # <ab|cd> t2_ijcd
        T_iakc = t2.permute(0, 2, 1, 3).reshape(nov, nov)                                # t2[i,k,a,c] as [(i,a),(k,c)]
        T_kcjb = t2.permute(0, 2, 1, 3).reshape(nov, nov)                                # t2[k,j,c,b] as [(k,c),(j,b)]
        T_x = t2.permute(0, 3, 1, 2).reshape(nov, nov)                                   # t2[i,k,c,a] as [(i,a),(k,c)]
        G_kcjb = self.g_ovvo.permute(0, 2, 3, 1).reshape(nov, nov)                       # <kb|cj> as [(k,c),(j,b)]
        W_kcjb = (2.0 * self.g_ovvo - self.g_ovov.permute(0, 1, 3, 2)).permute(0, 2, 3, 1).reshape(nov, nov)
        W_iakc = (2.0 * self.g_ovvo - self.g_ovov.permute(0, 1, 3, 2)).permute(3, 1, 0, 2).reshape(nov, nov)
        G_iakc = self.g_ovvo.permute(3, 1, 0, 2).reshape(nov, nov)                      # <ka|ci> as [(i,a),(k,c)]
        Gs_ibkc = self.g_ovov.permute(2, 1, 0, 3).reshape(nov, nov)                     # <kb|ic> as [(i,b),(k,c)]
        Gs_kcja = self.g_ovov.permute(0, 3, 2, 1).reshape(nov, nov)                     # <ka|jc> as [(k,c),(j,a)]
        T_kcja = t2.permute(0, 3, 1, 2).reshape(nov, nov)                                # t2[k,j,a,c] as [(k,c),(j,a)]
        T_kcjb2 = t2.permute(0, 3, 1, 2).reshape(nov, nov)                               # t2[k,j,b,c] as [(k,c),(j,b)]
        T_ibkc = t2.permute(0, 3, 1, 2).reshape(nov, nov)                                # t2[i,k,c,b] as [(i,b),(k,c)]
        iajb = lambda X: X.reshape(no, nv, no, nv).permute(0, 2, 1, 3)
        ibja = lambda X: X.reshape(no, nv, no, nv).permute(0, 2, 3, 1)
        r2 -= iajb(_mm(T_x, G_kcjb))                                                     # <kb|cj> t2_ikca
        r2 += iajb(_mm(W_iakc, T_kcjb))                                                  # (2<ka|ci> - <ka|ic>) t2_kjcb
        r2 -= ibja(_mm(Gs_ibkc, T_kcja))                                                 # <kb|ic> t2_kjac
        r2 -= iajb(_mm(G_iakc, T_kcjb2))                                                 # <ka|ci> t2_kjbc
        r2 += iajb(_mm(T_iakc, W_kcjb))                                                  # (2<kb|cj> - <kb|jc>) t2_ikac
        r2 -= ibja(_mm(T_ibkc, Gs_kcja))                                                 # <ka|jc> t2_ikcb
        r2 -= E * t2
        return r1, r2

    def energy(self, t1, t2):
        """2 t1.F_ov + t2.(2<ij|ab> - <ij|ba>), no conjugation (apyib/ci_wfn.py:510)."""
        E = bdot(t2.reshape(1, -1), self.L_oovv.reshape(1, -1))[0]
        if self.singles:
            E = E + 2.0 * bdot(t1.reshape(1, -1), self.Fov.reshape(1, -1))[0]
        return complex(E)

    # ------------------------------------------------------------------ solver
    def solve(self, params, print_level=0, history=None):
        """Jacobi + DIIS iteration of apyib/ci_wfn.py:420-535 (CISD) / :51-160 (CID).
        Returns (E, t1, t2) with t1 None for CID."""
        no, nv = self.no, self.nv
        t1 = (self.Fvo_T / self.D_ia).contiguous() if self.singles else None
        t2 = (self.g_vvoo.permute(2, 3, 0, 1) / self.D_ijab).contiguous()
        E = self.energy(t1, t2)
        n1 = no * nv if self.singles else 0
        e_hist, t_hist = [], []
        B = np.zeros((0, 0), dtype=np.complex128)
        it = 1
        while it <= params["max_iterations"]:
            E_old = E
            t1_old = None if t1 is None else t1.clone()
            t2_old = t2.clone()
            r1, r2 = self.residual(t1, t2, E)
            if self.singles:
                t1 = t1 + r1 / self.D_ia
            t2 = t2 + r2 / self.D_ijab
            if params["DIIS"]:
                res = r2.reshape(-1) if not self.singles else torch.cat((r1.reshape(-1), r2.reshape(-1)))
                tv = t2.reshape(-1) if not self.singles else torch.cat((t1.reshape(-1), t2.reshape(-1)))
                if it == 1:
                    e_hist, t_hist = [res], [tv]
                    B = np.array([[complex(bdot(res.conj().reshape(1, -1), res.reshape(1, -1))[0])]])
                else:
                    while len(e_hist) > 7:
                        e_hist.pop(0)
                        t_hist.pop(0)
                        B = B[1:, 1:]
                    ys = e_hist + [res]
                    Y = torch.stack(ys).conj()
                    d = bdot(Y, res.reshape(1, -1)).cpu().numpy()                 # conj(e_j) . res
                    m = len(e_hist)
                    Bn = np.zeros((m + 1, m + 1), dtype=np.complex128)
                    Bn[:m, :m] = B
                    Bn[:m, m] = d[:m]
                    Bn[m, :m] = np.conj(d[:m])
                    Bn[m, m] = d[m]
                    B = Bn
                    e_hist.append(res)
                    t_hist.append(tv)
                c = torch.as_tensor(_bordered_diis(B)).to(t2.device)
                tv = _mm(torch.stack(t_hist).T, c.reshape(-1, 1)).reshape(-1)
                if self.singles:
                    t1 = tv[:n1].reshape(no, nv).contiguous()
                t2 = tv[n1:].reshape(no, no, nv, nv).contiguous()
            E = self.energy(t1, t2)
            d2 = (t2_old - t2).reshape(1, -1)
            rms_t2 = np.sqrt(np.complex128(complex(bdot(d2, d2)[0])))
            rms_t1 = 0.0
            if self.singles:
                d1 = (t1_old - t1).reshape(1, -1)
                rms_t1 = np.sqrt(np.complex128(complex(bdot(d1, d1)[0])))
            dE = E_old - E
            if history is not None:
                history.append(dict(iteration=it, E=E, dE=dE, rms_t1=complex(rms_t1), rms_t2=complex(rms_t2)))
            if print_level > 0:
                print(" %02d %20.12f %20.12f %20.12f %20.12f" % (it, E.real, E.imag, dE.real, complex(rms_t2).real))
            if it > 1 and abs(dE) < params["e_convergence"] and _lt(rms_t2, params["d_convergence"]) and (
                    not self.singles or _lt(rms_t1, params["d_convergence"])):
                break
            if it == params["max_iterations"]:
                if abs(dE) > params["e_convergence"] or np.complex128(rms_t2) > params["d_convergence"]:
                    print("Not converged.")
            it += 1
        return E, t1, t2
