"""Hand-written adjoint of the spin-orbital CISD energy.

The CISD_SO energy of apyib/ci_wfn.py:263-378 is the eigenvalue of the
normal-ordered Hamiltonian in the singles+doubles space.  Its derivative
with respect to any one- or two-electron integral is therefore the
expectation value of the corresponding operator in the normalised CI state
(Hellmann-Feynman; no amplitude response is needed):

    dE = sum_pq D_pq dF_pq + sum_pqrs Gamma_pqrs d<pq|rs>

with the one- and two-particle densities of the reference's own adjoint
check (apyib/ci_wfn.py:382-411, restated in oracle/port.py), with one
change: the reference's doubles equations (ci_wfn.py:319-334) have no F_vo t1
coupling, so the eigenproblem the solver converges is not Hermitian once F_vo
is non-zero; its left eigenvector at a point with F_vo = 0 is still the
conjugate of the right one, and the derivative with respect to F_vo then
lacks the sum_jb t2*_ijab t1_jb term of the exact CISD density.  ``densities``
drops it by default (``vo_coupling=False``), which makes dE/dF exact for every
Fock block; the two agree whenever F_vo = 0.  The densities
are built on the GPU from the converged amplitudes with the library's
complex GEMMs; the vvvv block Gamma_abcd = 1/4 sum_ij t2*_ijab t2_ijcd is
recomputed in the backward as a packed (a<b, c<d) GEMM over i<j rather than
kept from the forward pass.

``CISDEnergy`` wraps the solve in a torch.autograd.Function with inputs
(F_SO, ERI_SO) (chemist, <pq|rs> = (pr|qs)); ``CISDEnergyCore`` takes the AO
core Hamiltonian h = T + V at fixed orbitals and returns dE/dh = C* D C^T,
the route to magnetic-field derivatives (dh/dB = -mu_mag) without orbital
relaxation.  Gradients follow PyTorch's convention for a holomorphic map:
grad_input = grad_output * conj(dE/dinput).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .cisd import CISDPlan, solve
from .device import device, ptr, stream_ptr, to_dev
from .linalg import zmm


def _zgemm_conjA(A_ptr_tensor, M, N, K, sAm, sAk, B, sBk, sBn, out, alpha=1.0, precision=_lib.PREC_FP64,
                 scratch=None):
    a = complex(alpha)
    if precision == _lib.PREC_TF32X3:
        buf, nb = scratch
        _lib.call("agb_cgemm_tf32x3", M, N, K, a.real, a.imag, ptr(A_ptr_tensor), sAm, sAk, 1, ptr(B), sBk, sBn, 0,
                  0.0, 0.0, ptr(out), N, ptr(buf), nb, stream_ptr())
    else:
        _lib.call("agb_zgemm", M, N, K, a.real, a.imag, ptr(A_ptr_tensor), sAm, sAk, 1, ptr(B), sBk, sBn, 0, 0.0, 0.0,
                  ptr(out), N, stream_ptr())


def densities(plan, t, precision=_lib.PREC_FP64, vo_coupling=False):
    """One- and two-particle densities of the normalised CISD_SO (or CID_SO)
    state from the packed amplitudes t.  Returns (D [nso,nso], G) with G a
    dict of Dirac-ordered blocks keyed by orbital-range letters; G['vvvv_p']
    is the packed block Gp[(a<b),(c<d)] with Gamma_abcd = sign * Gp / 2.

    vo_coupling=True gives the exact CISD density of apyib/ci_wfn.py:393
    (D_ai = t0 t1*_ia + sum_jb t2*_ijab t1_jb); the default drops the second
    term, which couples F_vo to the doubles - a coupling the reference's
    residual (ci_wfn.py:319-334) does not contain - so that D is the derivative
    of the energy the solver actually converges (identical when F_vo = 0)."""
    o, v = plan.o, plan.v
    nso = o + v
    dev = device()

    def mm(*a, **k):
        return zmm(*a, precision=precision, **k)

    t1, t2 = plan.unpack(t)
    if t1 is None:
        t1 = torch.zeros((o, v), dtype=torch.complex128, device=dev)
    n1 = torch.sum(t1.conj() * t1).real
    n2 = torch.sum(t2.conj() * t2).real
    N = float(1.0 / torch.sqrt(1.0 + n1 + 0.25 * n2))
    t0 = N
    t1 = t1 * N
    t2 = t2 * N
    t1c = t1.conj()
    O, V = slice(0, o), slice(o, nso)
    D = torch.zeros((nso, nso), dtype=torch.complex128, device=dev)
    T2m = t2.reshape(o, o * v * v)
    D[O, O] = -(mm(t1, t1, transB=True, conjB=True) + 0.5 * mm(T2m, T2m, transB=True, conjB=True))
    Tv = t2.permute(2, 0, 1, 3).reshape(v, o * o * v).contiguous()
    D[V, V] = mm(t1, t1, transA=True, conjA=True) + 0.5 * mm(Tv, Tv, conjA=True, transB=True)
    Tr = t2.permute(0, 2, 1, 3).reshape(o * v, o * v).contiguous()       # [(i,a),(j,b)] = t2[i,j,a,b]
    D[O, V] = t0 * t1 + mm(Tr, t1c.reshape(o * v, 1)).reshape(o, v)
    if vo_coupling:
        D[V, O] = (t0 * t1c + mm(Tr, t1.reshape(o * v, 1), conjA=True).reshape(o, v)).T
    else:
        D[V, O] = (t0 * t1c).T
    G = {}
    # oooo: 1/4 sum_ab t2*[k,l,a,b] t2[i,j,a,b] -> [i,j,k,l]
    Toov = t2.reshape(o * o, v * v)
    G["oooo"] = 0.25 * mm(Toov, Toov, transB=True, conjB=True).reshape(o, o, o, o)
    # ovvo / ovov from t1: 'ja,ib->iabj' and -'ja,ib->iajb'
    P = torch.einsum("ja,ib->iabj", t1c, t1)          # outer product (no contraction)
    G["ovvo"] = P.contiguous()
    G["ovov"] = (-P.permute(0, 1, 3, 2)).contiguous()
    # voov / vovo: 'jkac,ikbc->aijb' and -'jkac,ikbc->aibj'
    Tk = t2.permute(0, 2, 1, 3).reshape(o * v, o * v)   # [(j,a),(k,c)]
    Q = mm(Tk, Tk, conjA=True, transB=True).reshape(o, v, o, v)      # Q[j,a,i,b] = sum_kc t2*[jkac] t2[ikbc]
    G["voov"] = Q.permute(1, 2, 0, 3).contiguous()                    # [a,i,j,b]
    G["vovo"] = (-Q.permute(1, 2, 3, 0)).contiguous()                 # [a,i,b,j]
    G["oovv"] = 0.5 * t0 * t2
    G["vvoo"] = (0.5 * t0 * t2.conj().permute(2, 3, 0, 1)).contiguous()
    # vovv: 'ja,ijcb->aibc'
    G["vovv"] = mm(t1c, t2.permute(1, 0, 3, 2).reshape(o, o * v * v), transA=True).reshape(v, o, v, v)
    # ovoo: -'kjab,ib->iajk'
    Tb = t2.conj().permute(3, 2, 1, 0).reshape(v, v * o * o).contiguous()   # [b,(a,j,k)] = t2*[k,j,a,b]
    G["ovoo"] = (-mm(t1, Tb).reshape(o, v, o, o)).contiguous()             # X[i,(a,j,k)] = sum_b t1[i,b] Tb

    # vvvo: 'jiab,jc->abci'
    G["vvvo"] = mm(t2.conj().permute(2, 3, 1, 0).reshape(v * v * o, o), t1).reshape(v, v, o, v).permute(
        0, 1, 3, 2).contiguous()
    # ooov: -'kb,ijba->ijka'
    G["ooov"] = (-mm(t2.permute(0, 1, 3, 2).reshape(o * o * v, v), t1c, transB=True)
                 .reshape(o, o, v, o).permute(0, 1, 3, 2)).contiguous()
    # vvvv (packed, recomputed): Gp[(ab),(cd)] = sum_{i<j} t2p*[ij,ab] t2p[ij,cd]; Gamma = Gp/2 with signs
    n1v = plan.n1
    t2p = (t[n1v:] * N).contiguous()
    po, pv = o * (o - 1) // 2, v * (v - 1) // 2
    Gp = torch.empty((pv, pv), dtype=torch.complex128, device=dev)
    if precision == _lib.PREC_TF32X3:
        nb = _lib.load().agb_cgemm_tf32x3_scratch_bytes(pv, pv, po)
        buf = torch.zeros(int(nb) // 8 + 64, dtype=torch.float64, device=dev)
        _zgemm_conjA(t2p, pv, pv, po, 1, pv, t2p, pv, 1, Gp, precision=precision, scratch=(buf, nb))
    else:
        _zgemm_conjA(t2p, pv, pv, po, 1, pv, t2p, pv, 1, Gp)
    G["vvvv_p"] = Gp
    G["_norm"] = N
    return D, G


def unpack_vvvv(Gp, v):
    """Full Gamma_vvvv[a,b,c,d] from the packed block (Gamma = Gp/2 with antisymmetry signs)."""
    dev = Gp.device
    iu = torch.triu_indices(v, v, offset=1, device=dev)
    full = torch.zeros((v, v, v, v), dtype=Gp.dtype, device=dev)
    a, b = iu[0], iu[1]
    g = 0.5 * Gp
    A = a.view(-1, 1).expand(-1, a.numel())
    Bb = b.view(-1, 1).expand(-1, a.numel())
    C = a.view(1, -1).expand(a.numel(), -1)
    Dd = b.view(1, -1).expand(a.numel(), -1)
    full[A, Bb, C, Dd] = g
    full[Bb, A, C, Dd] = -g
    full[A, Bb, Dd, C] = -g
    full[Bb, A, Dd, C] = g
    return full


def gamma_full(G, o, v):
    """Assemble the full Dirac Gamma[p,q,r,s] (nso^4) from the blocks."""
    nso = o + v
    dev = next(x for x in G.values() if isinstance(x, torch.Tensor)).device
    Gm = torch.zeros((nso, nso, nso, nso), dtype=torch.complex128, device=dev)
    O, V = slice(0, o), slice(o, nso)
    m = {"o": O, "v": V}
    for k in ("oooo", "ovvo", "ovov", "voov", "vovo", "oovv", "vvoo", "vovv", "ovoo", "vvvo", "ooov"):
        if k in G:
            Gm[m[k[0]], m[k[1]], m[k[2]], m[k[3]]] += G[k]
    if "vvvv_p" in G:
        Gm[V, V, V, V] += unpack_vvvv(G["vvvv_p"], v)
    return Gm


def energy_from_densities(F, ERI_chem, D, Gfull):
    """E = sum F D + sum <pq|rs> Gamma with <pq|rs> = (pr|qs)."""
    dirac = ERI_chem.permute(0, 2, 1, 3)
    return torch.sum(F * D) + torch.sum(dirac * Gfull)


class CISDEnergy(torch.autograd.Function):
    """E_CISD_SO(F_SO, ERI_SO) with a density-based backward.  eps_o / eps_v
    (spatial, np.repeat-ed for the denominators) and params are constants."""

    @staticmethod
    def forward(ctx, F_SO, ERI_SO, eps_o, eps_v, params, singles=True, precision="fp64"):
        o, v = 2 * len(eps_o), 2 * len(eps_v)
        plan = CISDPlan(o, v, singles=singles, mixed=(precision == "mixed"))
        eps_so = np.concatenate([np.repeat(eps_o, 2), np.repeat(eps_v, 2)])
        plan.set_fock(F_SO.detach(), eps_so)
        plan.blocks_from_so(ERI_SO.detach())
        E, t = solve(plan, params, precision=precision)
        ctx.plan = plan
        ctx.o, ctx.v = o, v
        ctx.save_for_backward(t)
        return torch.tensor(complex(E), dtype=torch.complex128, device=F_SO.device)

    @staticmethod
    def backward(ctx, gE):
        (t,) = ctx.saved_tensors
        D, G = densities(ctx.plan, t)
        Gfull = gamma_full(G, ctx.o, ctx.v)
        g = gE.to(torch.complex128)
        grad_F = g * D.conj()
        # <pq|rs> = (pr|qs): d E / d (pr|qs) = Gamma[p,q,r,s]
        grad_ERI = g * Gfull.permute(0, 2, 1, 3).conj()
        return grad_F, grad_ERI, None, None, None, None, None


def cisd_energy(F_SO, ERI_SO, eps_o, eps_v, params, singles=True, precision="fp64"):
    return CISDEnergy.apply(to_dev(F_SO) if not isinstance(F_SO, torch.Tensor) else F_SO,
                            to_dev(ERI_SO) if not isinstance(ERI_SO, torch.Tensor) else ERI_SO,
                            eps_o, eps_v, params, singles, precision)


# ---------------------------------------------------------------------------
# MP2_SO: the Hylleraas Lagrangian and its densities
#
# The MP2_SO energy of apyib/mp2_wfn.py:64-87, E = 1/4 sum <ij||ab> t_ijab with
# t_ijab = <ab||ij> / D_ijab (no conjugate), is the stationary value of
#     L(t, lam) = 1/4 <W, t> + 1/4 <lam, V + A t>,    <x, y> = sum_ijab x_ijab y_ijab,
# W_ijab = <ij||ab>, V_ijab = <ab||ij>, and A the Fock operator on the doubles,
#     (A t)_ijab = sum_c (F_bc t_ijac + F_ac t_ijcb) - sum_k (F_kj t_ikab + F_ki t_kjab),
# whose diagonal part is -D t (D_ijab = F_ii + F_jj - F_aa - F_bb; the reference's
# orbital energies when F is the canonical Fock matrix).  Stationarity gives the
# amplitude equations V + A t = 0 and the left equations W + A^T lam = 0 (A^T: F
# transposed), so lam = W / D at a canonical point, lam = conj(t) for Hermitian
# integrals.  The derivatives of L are densities in the format of ``densities``:
#     D_oo[x,y] = -1/2 sum_iab t_ixab lam_iyab,   D_vv[x,y] = 1/2 sum_ija lam_ijax t_ijay,
#     Gamma_oovv = t / 2,   Gamma_vvoo[a,b,i,j] = lam_ijab / 2,
# and E = sum F D + sum <pq|rs> Gamma holds at the solution.  With a non-canonical F
# (off-diagonal occupied-occupied or virtual-virtual elements) the amplitudes solve
# the full equations, the non-canonical MP2 that apyib/analytic_aats.py:215-549
# differentiates for its MP2 AATs.

def mp2_fock_apply(t, Fo, Fv, transpose=False):
    """(A t)_ijab = sum_c (F_bc t_ijac + F_ac t_ijcb) - sum_k (F_kj t_ikab + F_ki t_kjab) for
    antisymmetric t[o,o,v,v] and the given occupied / virtual Fock blocks (F^T with
    transpose=True), on the library's complex GEMM."""
    o, v = t.shape[0], t.shape[2]
    if transpose:
        Fo, Fv = Fo.T.contiguous(), Fv.T.contiguous()
    X = zmm(t.reshape(o * o * v, v), Fv, transB=True).reshape(o, o, v, v)     # sum_c F_bc t_ijac
    Tk = t.permute(1, 0, 2, 3).reshape(o, o * v * v).contiguous()
    Z = zmm(Fo, Tk, transA=True).reshape(o, o, v, v).permute(1, 0, 2, 3)      # sum_k F_kj t_ikab
    return (X - X.transpose(2, 3)) - (Z - Z.transpose(0, 1))


def _mp2_fock_offdiag(t, Foo, Fvv, transpose=False):
    """The off-diagonal part of (A t) (or A^T t)."""
    return mp2_fock_apply(t, Foo - torch.diag(torch.diagonal(Foo)), Fvv - torch.diag(torch.diagonal(Fvv)),
                          transpose=transpose)


def _mp2_denominators(Foo, Fvv):
    eo, ev = torch.diagonal(Foo), torch.diagonal(Fvv)
    return eo.view(-1, 1, 1, 1) + eo.view(1, -1, 1, 1) - ev.view(1, 1, -1, 1) - ev.view(1, 1, 1, -1)


def mp2_so_blocks(ERI_SO, o):
    """W[i,j,a,b] = <ij||ab> and V[i,j,a,b] = <ab||ij> from a chemist spin-orbital tensor
    (<pq|rs> = (pr|qs)), gathered on the device."""
    g = ERI_SO
    O, V = slice(0, o), slice(o, g.shape[0])
    ovov = g[O, V, O, V]
    vovo = g[V, O, V, O]
    W = ovov.permute(0, 2, 1, 3) - ovov.permute(0, 2, 3, 1)
    Vb = vovo.permute(1, 3, 0, 2) - vovo.permute(3, 1, 0, 2)
    return W.contiguous(), Vb.contiguous()


def mp2_lagrangian_solve(F_SO, W, V, o, tol=1e-14, max_iterations=200):
    """Amplitudes t and multipliers lam of the MP2_SO Lagrangian for the Fock matrix
    F_SO (its occupied-occupied and virtual-virtual blocks) and the blocks W, V of
    ``mp2_so_blocks``: t = (V + A_off t) / D and lam = (W + A_off^T lam) / D by
    Jacobi iteration (one step when F is diagonal).  Returns (E, t, lam)."""
    Foo, Fvv = F_SO[:o, :o], F_SO[o:, o:]
    D = _mp2_denominators(Foo, Fvv)
    offdiag = bool((Foo - torch.diag(torch.diagonal(Foo))).abs().max() > 0 or
                   (Fvv - torch.diag(torch.diagonal(Fvv))).abs().max() > 0)
    out = []
    for rhs, tr in ((V, False), (W, True)):
        x = rhs / D
        if offdiag:
            for _ in range(max_iterations):
                xn = (rhs + _mp2_fock_offdiag(x, Foo, Fvv, transpose=tr)) / D
                step = (xn - x).abs().max().item()
                x = xn
                if step < tol * max(1.0, x.abs().max().item()):
                    break
            else:
                raise RuntimeError("non-canonical MP2 amplitudes did not converge")
        out.append(x)
    t, lam = out
    E = 0.25 * torch.sum(W * t)
    return complex(E), t, lam


def mp2_densities(t, lam):
    """Densities of the MP2_SO Lagrangian (see above) in the format of ``densities``:
    D (nso x nso; occupied-occupied and virtual-virtual blocks) and G with the oovv and
    vvoo Dirac blocks."""
    o, v = t.shape[0], t.shape[2]
    nso = o + v
    D = torch.zeros((nso, nso), dtype=torch.complex128, device=t.device)
    To = t.permute(1, 0, 2, 3).reshape(o, o * v * v).contiguous()
    Lo = lam.permute(1, 0, 2, 3).reshape(o, o * v * v).contiguous()
    D[:o, :o] = -0.5 * zmm(To, Lo, transB=True)
    D[o:, o:] = 0.5 * zmm(lam.reshape(o * o * v, v), t.reshape(o * o * v, v), transA=True)
    G = {"oovv": 0.5 * t, "vvoo": (0.5 * lam.permute(2, 3, 0, 1)).contiguous()}
    return D, G


class MP2Energy(torch.autograd.Function):
    """E_MP2_SO(F_SO, ERI_SO) (chemist ERIs) with the Lagrangian backward: dE/dF = D,
    dE/d<pq|rs> = Gamma (oo, vv and oovv / vvoo blocks).  At a diagonal F the energy is
    the reference's MP2_SO energy with the diagonal as orbital energies."""

    @staticmethod
    def forward(ctx, F_SO, ERI_SO, o):
        F = F_SO.detach().to(torch.complex128)
        W, V = mp2_so_blocks(ERI_SO.detach().to(torch.complex128), o)
        E, t, lam = mp2_lagrangian_solve(F, W, V, o)
        ctx.save_for_backward(t, lam)
        return torch.tensor(E, dtype=torch.complex128, device=F_SO.device)

    @staticmethod
    def backward(ctx, gE):
        t, lam = ctx.saved_tensors
        o, v = t.shape[0], t.shape[2]
        D, G = mp2_densities(t, lam)
        Gfull = gamma_full(G, o, v)
        g = gE.to(torch.complex128)
        return g * D.conj(), g * Gfull.permute(0, 2, 1, 3).conj(), None


def mp2_energy(F_SO, ERI_SO, o):
    """Differentiable MP2_SO energy (see MP2Energy)."""
    return MP2Energy.apply(to_dev(F_SO) if not isinstance(F_SO, torch.Tensor) else F_SO,
                           to_dev(ERI_SO) if not isinstance(ERI_SO, torch.Tensor) else ERI_SO, int(o))


# ---------------------------------------------------------------------------
# AO-level adjoint for the core Hamiltonian (field derivatives at fixed orbitals)

def _fock_mo(h_AO, ERI_AO, C, C_list, freeze_core):
    """F_MO = C_t^H (h + G[D_fc] + G[D_occ]) C_t with G[D] = 2J - K (apyib/utils.py:231-252)."""
    from .linalg import jk_fock
    f, o, _, t = C_list
    h = h_AO
    if freeze_core:
        Cf = C[:, f].contiguous()
        h = jk_fock(ERI_AO, zmm(Cf, Cf, transB=True, conjB=True), h, 1.0)
    Co = C[:, o].contiguous()
    F_AO = jk_fock(ERI_AO, zmm(Co, Co, transB=True, conjB=True), h, 1.0)
    Ct = C[:, t].contiguous()
    return zmm(zmm(Ct, F_AO, transA=True, conjA=True), Ct)


class CISDEnergyCore(torch.autograd.Function):
    """E_CISD_SO as a function of the AO core Hamiltonian h = T + V (complex),
    at fixed orbitals C (the wavefunction object's) and fixed AO ERIs.
    dE/dh = conj(C_t) D_sp C_t^T with D_sp the spin-summed active-space density,
    so dE/dB = Re sum conj(grad_h) dh/dB for a field term dh/dB = -mu_mag."""

    @staticmethod
    def forward(ctx, h_AO, wfn, params, precision="fp64"):
        from .utils import compute_ERI_MO, compute_F_SO, get_slices
        C_list, _ = get_slices(params, wfn)
        C = to_dev(np.asarray(wfn.C))
        ERI = to_dev(wfn.H.ERI, torch.float64)
        F_MO = _fock_mo(h_AO.detach(), ERI, C, C_list, params["freeze_core"])
        ERI_MO = compute_ERI_MO(params, wfn, C_list, return_torch=True)
        eps = np.asarray(wfn.eps)
        eps_o, eps_v = eps[C_list[1]], eps[C_list[2]]
        o, v = 2 * len(eps_o), 2 * len(eps_v)
        plan = CISDPlan(o, v, singles=params["method"] in ("CISD", "CISD_SO"), mixed=(precision == "mixed"))
        eps_so = np.concatenate([np.repeat(eps_o, 2), np.repeat(eps_v, 2)])
        plan.set_fock(compute_F_SO(wfn, F_MO, return_torch=True), eps_so)
        plan.blocks_from_mo(ERI_MO)
        E, t = solve(plan, params, precision=precision)
        ctx.plan = plan
        ctx.Ct = C[:, C_list[3]].contiguous()
        ctx.save_for_backward(t)
        return torch.tensor(complex(E), dtype=torch.complex128, device=h_AO.device)

    @staticmethod
    def backward(ctx, gE):
        (t,) = ctx.saved_tensors
        D, _ = densities(ctx.plan, t)
        D_sp = D[0::2, 0::2] + D[1::2, 1::2]            # F_SO[p,q] = F_MO[p/2,q/2] for equal spins
        Ct = ctx.Ct
        dEdh = zmm(zmm(Ct.conj().resolve_conj(), D_sp), Ct, transB=True)   # conj(C) D_sp C^T
        return gE.to(torch.complex128) * dEdh.conj(), None, None, None


def cisd_energy_core(h_AO, wfn, params, precision="fp64"):
    return CISDEnergyCore.apply(h_AO, wfn, params, precision)


# ---------------------------------------------------------------------------
# Gradient with respect to the MO coefficients (orbital-response right-hand side)

def _spin_summed(D, G, o, v):
    """Spatial densities of the SO ones (alpha even, beta odd): E = sum_PQ F_MO[P,Q] D_sp[P,Q]
    + sum_PQRS (PQ|RS)_MO Gc[P,Q,R,S], with (PR|QS) = <PQ|RS> for equal spins on P,R and Q,S."""
    D_sp = D[0::2, 0::2] + D[1::2, 1::2]
    Gd = gamma_full(G, o, v)
    n = (o + v) // 2
    Gc = torch.zeros((n, n, n, n), dtype=torch.complex128, device=Gd.device)
    for s1 in (0, 1):
        for s2 in (0, 1):
            Gc += Gd[s1::2, s2::2, s1::2, s2::2].permute(0, 2, 1, 3)
    return D_sp, Gc


def _back(X, Cm, axis):
    """Replace the MO index `axis` of X by an AO index: out[..m..] = sum_P Cm[m,P] X[..P..]."""
    Xp = X.movedim(axis, 0)
    rest = tuple(Xp.shape[1:])
    out = zmm(Cm, Xp.reshape(Xp.shape[0], -1).contiguous())
    return out.reshape((Cm.shape[0],) + rest).movedim(0, axis).contiguous()


def _contract3(T, H, axis):
    """X[a,P] = sum over the other three AO indices of T[...a...] H[...P...] (index `axis`)."""
    Tm = T.movedim(axis, 0).reshape(T.shape[axis], -1).contiguous()
    Hm = H.movedim(axis, 0).reshape(H.shape[axis], -1).contiguous()
    return zmm(Tm, Hm, transB=True)


def mo_coefficient_gradient(h_AO, wfn, params, precision="fp64", return_intermediates=False):
    """Wirtinger derivatives (E, dE/dC, dE/dC*) of the CISD_SO (CID_SO, or MP2_SO through
    its Lagrangian densities, ``mp2_densities``) correlation energy with
    respect to the MO coefficients C (nbf x nbf), at fixed AO integrals and fixed
    orbital energies, with C entering through F_MO = C_t^H (h + G[C_fc C_fc^H] +
    G[C_o C_o^H]) C_t and (PQ|RS) = sum C*_mP C_nQ C*_lR C_sS (mn|ls) (apyib/utils.py:
    217-279).  A first-order change dC gives dE = sum(dE/dC * dC) + sum(dE/dC* * conj(dC)):
    the right-hand side of an orbital-response (Z-vector) equation.  Uses the
    Hellmann-Feynman densities of the converged amplitudes (apyib/ci_wfn.py:382-411)
    and the 8-fold symmetry of the real AO integrals."""
    from .linalg import jk_fock
    from .utils import compute_ERI_MO, compute_F_SO, get_slices
    C_list, _ = get_slices(params, wfn)
    f, oc, _, t = C_list
    C = to_dev(np.asarray(wfn.C))
    ERI = to_dev(wfn.H.ERI, torch.float64)
    h = h_AO.detach() if isinstance(h_AO, torch.Tensor) else to_dev(h_AO)
    F_MO = _fock_mo(h, ERI, C, C_list, params["freeze_core"])
    ERI_MO = compute_ERI_MO(params, wfn, C_list, return_torch=True)
    eps = np.asarray(wfn.eps)
    eps_o, eps_v = eps[C_list[1]], eps[C_list[2]]
    o, v = 2 * len(eps_o), 2 * len(eps_v)
    eps_so = np.concatenate([np.repeat(eps_o, 2), np.repeat(eps_v, 2)])
    if params["method"] in ("MP2", "MP2_SO"):
        # MP2_SO amplitudes t = <ab||ij> / D (canonical orbitals); the Lagrangian's
        # multipliers lam = <ij||ab> / D = conj(t) for the Hermitian MO integrals
        plan = CISDPlan(o, v, mp2_only=True)
        plan.set_fock(compute_F_SO(wfn, F_MO, return_torch=True), eps_so)
        plan.blocks_from_mo(ERI_MO)
        E, tamp = plan.mp2()
        _, t2 = plan.unpack(tamp)
        D, G = mp2_densities(t2, t2.conj().resolve_conj())
    else:
        plan = CISDPlan(o, v, singles=params["method"] in ("CISD", "CISD_SO"), mixed=(precision == "mixed"))
        plan.set_fock(compute_F_SO(wfn, F_MO, return_torch=True), eps_so)
        plan.blocks_from_mo(ERI_MO)
        E, tamp = solve(plan, params, precision=precision)
        D, G = densities(plan, tamp)
    D_sp, Gc = _spin_summed(D, G, o, v)
    nbf = C.shape[0]
    Ct = C[:, t].contiguous()
    Ctc = Ct.conj().resolve_conj().contiguous()
    # F_AO at C (h + G[D_fc] + G[D_occ])
    hf = h
    if params["freeze_core"]:
        Cf = C[:, f].contiguous()
        hf = jk_fock(ERI, zmm(Cf, Cf, transB=True, conjB=True), h, 1.0)
    Co = C[:, oc].contiguous()
    F_AO = jk_fock(ERI, zmm(Co, Co, transB=True, conjB=True), hf, 1.0)
    dC = torch.zeros((nbf, nbf), dtype=torch.complex128, device=C.device)
    dCc = torch.zeros_like(dC)
    # through the MO transform of the Fock matrix
    dC[:, t] += zmm(zmm(F_AO, Ctc, transA=True), D_sp)
    dCc[:, t] += zmm(zmm(F_AO, Ct), D_sp, transB=True)
    # through the occupied (and frozen-core) densities inside F_AO: W = dE/dD_AO
    Y = zmm(zmm(Ctc, D_sp), Ct, transB=True)
    W = jk_fock(ERI, Y, torch.zeros_like(Y), 1.0)
    dC[:, oc] += zmm(W, Co.conj().resolve_conj())
    dCc[:, oc] += zmm(W, Co, transA=True)
    if params["freeze_core"]:
        dC[:, f] += zmm(W, Cf.conj().resolve_conj())
        dCc[:, f] += zmm(W, Cf, transA=True)
    # through the four-index transform: one index left in MO, three back-transformed
    T = ERI.to(torch.complex128)
    H1 = _back(_back(_back(Gc, Ct, 1), Ctc, 2), Ct, 3)      # [P, n, l, s]
    dCc[:, t] += _contract3(T, H1, 0)
    H2 = _back(_back(_back(Gc, Ctc, 0), Ctc, 2), Ct, 3)     # [m, Q, l, s]
    dC[:, t] += _contract3(T, H2, 1)
    H3 = _back(_back(_back(Gc, Ctc, 0), Ct, 1), Ct, 3)      # [m, n, R, s]
    dCc[:, t] += _contract3(T, H3, 2)
    H4 = _back(_back(_back(Gc, Ctc, 0), Ct, 1), Ctc, 2)     # [m, n, l, S]
    dC[:, t] += _contract3(T, H4, 3)
    if return_intermediates:
        # AO densities of the correlation energy at fixed orbitals: dE = sum Y dF_AO + sum G_AO d(mn|ls)
        G_AO = _back(H4, Ct, 3)
        return complex(E), dC, dCc, {"Y": Y, "G_AO": G_AO, "Co": Co, "Cf": Cf if params["freeze_core"] else None}
    return complex(E), dC, dCc
