"""CPU restatement (NumPy) of the Gaussian AO integrals apyib takes from psi4.

TEST INFRASTRUCTURE ONLY: the integral tests, ``smoke()`` and the CPU leg of
``bench.py`` use it as the checker; ``apyib_gb300`` never imports it.

Shells are ``(l, center[3], exps[n], coefs[n])`` with coefficients already
carrying the primitive normalisation; Cartesian components are ordered
``for i in 0..l: for j in 0..i: (l-i, i-j, j)`` (apyib/integrals.py:107-119).

* overlap, kinetic, dipole, nabla, angular momentum: the one-dimensional
  Obara-Saika tables and component products of apyib/integrals.py:63-141,
  with the sign conventions of :143-146 (dipole and angular momentum carry the
  electron charge, -1; kinetic is -1/2 nabla^2), origin 0;
* nuclear attraction and electron repulsion (psi4's ao_potential / ao_eri,
  apyib/hamiltonian.py:32-34, no reference code): McMurchie-Davidson Hermite
  expansion (McMurchie and Davidson, J. Comput. Phys. 26, 218 (1978)) with the
  Boys function from the regularised incomplete gamma function.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import gamma as _gamma
from scipy.special import gammainc


def cart(l):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def boys(nmax, T):
    """F_n(T) = int_0^1 t^(2n) exp(-T t^2) dt for n = 0..nmax; T an array."""
    T = np.asarray(T, dtype=np.float64)
    out = np.empty((nmax + 1,) + T.shape)
    small = T < 1e-12
    Ts = np.where(small, 1.0, T)
    for n in range(nmax + 1):
        a = n + 0.5
        v = _gamma(a) * gammainc(a, Ts) / (2.0 * Ts ** a)
        out[n] = np.where(small, 1.0 / (2 * n + 1) - T / (2 * n + 3), v)
    return out


# ----------------------------------------------------------------------------- one-electron (Obara-Saika)
def _os_table(la, lb, a, b, A, B):
    """S[alpha][i][j] for one primitive pair, i <= la, j <= lb
    (apyib/integrals.py:90-105)."""
    p = a + b
    mu = a * b / p
    P = (a * A + b * B) / p
    S = np.zeros((3, la + 1, lb + 1))
    for al in range(3):
        XPA, XPB, XAB = P[al] - A[al], P[al] - B[al], A[al] - B[al]
        S[al, 0, 0] = math.sqrt(math.pi / p) * math.exp(-mu * XAB * XAB)
        for i in range(la):
            S[al, i + 1, 0] = XPA * S[al, i, 0] + (i * S[al, i - 1, 0] if i > 0 else 0.0) / (2 * p)
        for i in range(la + 1):
            for j in range(lb):
                S[al, i, j + 1] = XPB * S[al, i, j] + ((i * S[al, i - 1, j] if i > 0 else 0.0)
                                                       + (j * S[al, i, j - 1] if j > 0 else 0.0)) / (2 * p)
    return S


def one_electron(shells, kind):
    """kind in {'overlap','kinetic','dipole','nabla','angular momentum'}; returns
    (n, n) or (3, n, n) over Cartesian functions (apyib/integrals.py:9-146)."""
    offs, n = [], 0
    for sh in shells:
        offs.append(n)
        n += len(cart(sh[0]))
    three = kind in ("dipole", "nabla", "angular momentum", "kinetic")
    M = np.zeros((3, n, n)) if three else np.zeros((n, n))
    for sa, (la, A, ea, ca) in enumerate(shells):
        A = np.asarray(A, dtype=np.float64)
        for sb, (lb, B, eb, cb) in enumerate(shells):
            B = np.asarray(B, dtype=np.float64)
            for a, c_a in zip(ea, ca):
                for b, c_b in zip(eb, cb):
                    S = _os_table(la + 1, lb + 2, a, b, A, B)

                    def s1(al, i, j):
                        return S[al, i, j] if i >= 0 and j >= 0 else 0.0

                    def mom(al, i, j):          # <i| x_al |j> with the origin at 0
                        return s1(al, i + 1, j) + A[al] * s1(al, i, j)

                    def der(al, i, j):          # <i| d/dx_al |j>
                        return j * s1(al, i, j - 1) - 2.0 * b * s1(al, i, j + 1)

                    def lap(al, i, j):          # <i| d^2/dx_al^2 |j>
                        return (j * (j - 1) * s1(al, i, j - 2) - 2.0 * b * (2 * j + 1) * s1(al, i, j)
                                + 4.0 * b * b * s1(al, i, j + 2))
                    cc = c_a * c_b
                    for ka, pa in enumerate(cart(la)):
                        for kb, pb in enumerate(cart(lb)):
                            I, J = offs[sa] + ka, offs[sb] + kb
                            sx, sy, sz = (s1(k, pa[k], pb[k]) for k in range(3))
                            if kind == "overlap":
                                M[I, J] += cc * sx * sy * sz
                                continue
                            ss = (sx, sy, sz)
                            for al in range(3):
                                o1, o2 = (al + 1) % 3, (al + 2) % 3
                                if kind == "dipole":
                                    v = mom(al, pa[al], pb[al]) * ss[o1] * ss[o2]
                                elif kind == "nabla":
                                    v = der(al, pa[al], pb[al]) * ss[o1] * ss[o2]
                                elif kind == "kinetic":
                                    v = lap(al, pa[al], pb[al]) * ss[o1] * ss[o2]
                                else:                   # (r x nabla)_al = r_o1 d_o2 - r_o2 d_o1
                                    v = ss[al] * (mom(o1, pa[o1], pb[o1]) * der(o2, pa[o2], pb[o2])
                                                  - mom(o2, pa[o2], pb[o2]) * der(o1, pa[o1], pb[o1]))
                                M[al, I, J] += cc * v
    if kind in ("dipole", "angular momentum"):
        M = -M
    if kind == "kinetic":
        M = -0.5 * M.sum(axis=0)
    return M


# ----------------------------------------------------------------------------- McMurchie-Davidson
def _hermite_E(la, lb, a, b, XAB):
    """E[i, j, t, ...] Hermite expansion coefficients of x_A^i x_B^j for primitive
    exponent arrays a, b (broadcast)."""
    p = a + b
    XPA = -b * XAB / p
    XPB = a * XAB / p
    shape = np.broadcast(a, b).shape
    E = np.zeros((la + 1, lb + 1, la + lb + 2) + shape)
    E[0, 0, 0] = np.exp(-(a * b / p) * XAB * XAB)
    h = 0.5 / p
    for i in range(la + 1):
        for j in range(lb + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                src, X = E[i - 1, j], XPA
            else:
                src, X = E[i, j - 1], XPB
            for t in range(i + j + 1):
                v = X * src[t]
                if t > 0:
                    v = v + h * src[t - 1]
                v = v + (t + 1) * src[t + 1]
                E[i, j, t] = v
    return E


def _hermite_R(L, alpha, XPC, YPC, ZPC):
    """R[t, u, v, ...] = R^0_tuv for t + u + v <= L."""
    T = alpha * (XPC * XPC + YPC * YPC + ZPC * ZPC)
    F = boys(L, T)
    shape = np.shape(T)
    cur = None
    for n in range(L, -1, -1):
        new = np.zeros((L + 1, L + 1, L + 1) + shape)
        new[0, 0, 0] = (-2.0 * alpha) ** n * F[n]
        m = L - n
        for t in range(m + 1):
            for u in range(m + 1 - t):
                for v in range(m + 1 - t - u):
                    if t + u + v == 0:
                        continue
                    if t > 0:
                        val = XPC * cur[t - 1, u, v] + ((t - 1) * cur[t - 2, u, v] if t > 1 else 0.0)
                    elif u > 0:
                        val = YPC * cur[t, u - 1, v] + ((u - 1) * cur[t, u - 2, v] if u > 1 else 0.0)
                    else:
                        val = ZPC * cur[t, u, v - 1] + ((v - 1) * cur[t, u, v - 2] if v > 1 else 0.0)
                    new[t, u, v] = val
        cur = new
    return cur


def potential(shells, charges, centers):
    """V_ab = -sum_C Z_C <a| 1/|r - C| |b> over Cartesian functions."""
    offs, n = [], 0
    for sh in shells:
        offs.append(n)
        n += len(cart(sh[0]))
    V = np.zeros((n, n))
    centers = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
    for sa, (la, A, ea, ca) in enumerate(shells):
        A = np.asarray(A, dtype=np.float64)
        for sb, (lb, B, eb, cb) in enumerate(shells):
            B = np.asarray(B, dtype=np.float64)
            a = np.asarray(ea)[:, None]
            b = np.asarray(eb)[None, :]
            p = a + b
            cc = np.asarray(ca)[:, None] * np.asarray(cb)[None, :]
            P = [(a * A[k] + b * B[k]) / p for k in range(3)]
            E = [_hermite_E(la, lb, a, b, A[k] - B[k]) for k in range(3)]
            for Zc, C in zip(charges, centers):
                R = _hermite_R(la + lb, p, P[0] - C[0], P[1] - C[1], P[2] - C[2])
                pre = -Zc * 2.0 * math.pi / p * cc
                for ka, pa in enumerate(cart(la)):
                    for kb, pb in enumerate(cart(lb)):
                        acc = 0.0
                        for t in range(pa[0] + pb[0] + 1):
                            for u in range(pa[1] + pb[1] + 1):
                                for v in range(pa[2] + pb[2] + 1):
                                    acc = acc + E[0][pa[0], pb[0], t] * E[1][pa[1], pb[1], u] * \
                                        E[2][pa[2], pb[2], v] * R[t, u, v]
                        V[offs[sa] + ka, offs[sb] + kb] += float(np.sum(pre * acc))
    return V


def eri(shells):
    """(ab|cd) over Cartesian functions, chemist order, full n^4 array."""
    offs, n = [], 0
    for sh in shells:
        offs.append(n)
        n += len(cart(sh[0]))
    G = np.zeros((n, n, n, n))
    ns = len(shells)
    pairs = {}
    for s1 in range(ns):
        for s2 in range(ns):
            la, A, ea, ca = shells[s1]
            lb, B, eb, cb = shells[s2]
            A = np.asarray(A, dtype=np.float64)
            B = np.asarray(B, dtype=np.float64)
            a = np.repeat(np.asarray(ea, dtype=np.float64), len(eb))
            b = np.tile(np.asarray(eb, dtype=np.float64), len(ea))
            c = np.repeat(np.asarray(ca, dtype=np.float64), len(eb)) * np.tile(np.asarray(cb, dtype=np.float64), len(ea))
            p = a + b
            P = np.stack([(a * A[k] + b * B[k]) / p for k in range(3)])
            E = [_hermite_E(la, lb, a, b, A[k] - B[k]) for k in range(3)]
            pairs[s1, s2] = (la, lb, p, P, c, E)
    for s1 in range(ns):
        for s2 in range(s1 + 1):
            for s3 in range(ns):
                for s4 in range(s3 + 1):
                    if (s3, s4) > (s1, s2):
                        continue
                    la, lb, p, P, c1, E1 = pairs[s1, s2]
                    lc, ld, q, Q, c2, E2 = pairs[s3, s4]
                    L = la + lb + lc + ld
                    pp = p[:, None]
                    qq = q[None, :]
                    alpha = pp * qq / (pp + qq)
                    R = _hermite_R(L, alpha, P[0][:, None] - Q[0][None, :], P[1][:, None] - Q[1][None, :],
                                   P[2][:, None] - Q[2][None, :])
                    pre = 2.0 * math.pi ** 2.5 / (pp * qq * np.sqrt(pp + qq)) * c1[:, None] * c2[None, :]
                    for ka, pa in enumerate(cart(la)):
                        for kb, pb in enumerate(cart(lb)):
                            for kc, pc in enumerate(cart(lc)):
                                for kd, pd in enumerate(cart(ld)):
                                    acc = 0.0
                                    for t in range(pa[0] + pb[0] + 1):
                                        for u in range(pa[1] + pb[1] + 1):
                                            for v in range(pa[2] + pb[2] + 1):
                                                e1 = (E1[0][pa[0], pb[0], t] * E1[1][pa[1], pb[1], u]
                                                      * E1[2][pa[2], pb[2], v])[:, None]
                                                for tt in range(pc[0] + pd[0] + 1):
                                                    for uu in range(pc[1] + pd[1] + 1):
                                                        for vv in range(pc[2] + pd[2] + 1):
                                                            e2 = (E2[0][pc[0], pd[0], tt] * E2[1][pc[1], pd[1], uu]
                                                                  * E2[2][pc[2], pd[2], vv])[None, :]
                                                            sgn = -1.0 if (tt + uu + vv) % 2 else 1.0
                                                            acc = acc + sgn * e1 * e2 * R[t + tt, u + uu, v + vv]
                                    val = float(np.sum(pre * acc))
                                    i, j = offs[s1] + ka, offs[s2] + kb
                                    k, l = offs[s3] + kc, offs[s4] + kd
                                    for (w, x, y, z) in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                                                         (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                                        G[w, x, y, z] = val
    return G


def shells_of(basis):
    """(l, center, exps, coefs) tuples from an object with ``.shells`` whose items
    have ``l, center, exps, coefs``."""
    return [(sh.l, np.asarray(sh.center), np.asarray(sh.exps), np.asarray(sh.coefs)) for sh in basis.shells]
