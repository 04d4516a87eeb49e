"""CPU restatement of the finite-difference AAT determinant sums (apyib/aats.py:120-555).

TEST INFRASTRUCTURE ONLY (the oracle).  Every overlap between excited
determinants is evaluated as the reference does: swap rows (bra excitation
i <-> a, j <-> b) and columns (ket excitation) of the spin-orbital MO overlap
and take the determinant of the occupied block (apyib/aats.py:120-131), one
determinant per excitation pair, with weights 1 (singles) and 1/4 (doubles);
the terms I_00 ... I_DS and the normalisations follow apyib/aats.py:134-555.
Spatial amplitudes are expanded to spin orbitals first.  Cost O((ov)^4 o^3):
small systems only.
"""
from __future__ import annotations

import numpy as np


def swap_det(S, o, bra, ket):
    """apyib/aats.py:120-131."""
    S = S.copy()
    for x in range(0, len(bra), 2):
        S[[bra[x], bra[x + 1]], :] = S[[bra[x + 1], bra[x]], :]
    for y in range(0, len(ket), 2):
        S[:, [ket[y], ket[y + 1]]] = S[:, [ket[y + 1], ket[y]]]
    return np.linalg.det(S[:o, :o])


def _excitations(rank, amp, o, f, nso):
    """(weight * amplitude, swap list) over all excitations of a rank."""
    if rank == 0:
        return [(1.0, [])]
    out = []
    occ, vir = range(f, o), range(o, nso)
    if rank == 1:
        for i in occ:
            for a in vir:
                w = amp[i - f, a - o]
                if w != 0:
                    out.append((w, [i, a]))
    else:
        for i in occ:
            for a in vir:
                for j in occ:
                    for b in vir:
                        w = amp[i - f, j - f, a - o, b - o]
                        if w != 0:
                            out.append((0.25 * w, [i, a, j, b]))
    return out


def _swapped(rank, amp, o, f, nso):
    """Weights and occupied row (or column) index lists of every excitation, the
    index list made by the same sequence of swaps as apyib/aats.py:124-127."""
    ws, idx = [], []
    for w, sw in _excitations(rank, amp, o, f, nso):
        p = np.arange(nso)
        for x in range(0, len(sw), 2):
            p[[sw[x], sw[x + 1]]] = p[[sw[x + 1], sw[x]]]
        ws.append(w)
        idx.append(p[:o])
    return np.array(ws, dtype=complex), np.array(idx)


def q(S, o, f, r, x, s, y):
    """sum over bra/ket excitations of weight * det(swapped occupied block)
    (determinants batched, in chunks of bra excitations)."""
    nso = S.shape[0]
    wx, rows = _swapped(r, x, o, f, nso)
    wy, cols = _swapped(s, y, o, f, nso)
    tot = 0.0
    step = max(1, int(2e6 // max(1, len(wy) * o * o)))
    for c0 in range(0, len(wx), step):
        blocks = S[rows[c0:c0 + step, None, :, None], cols[None, :, None, :]]
        tot += wx[c0:c0 + step] @ np.linalg.det(blocks) @ wy
    return tot


def so_amplitudes(t1, t2):
    """Closed-shell spatial amplitudes -> spin orbitals (alpha even, beta odd)."""
    o, _, v, _ = t2.shape
    T2 = np.zeros((2 * o, 2 * o, 2 * v, 2 * v), dtype=complex)
    tba = t2.transpose(0, 1, 3, 2)
    T2[0::2, 1::2, 0::2, 1::2] = t2
    T2[1::2, 0::2, 1::2, 0::2] = t2
    T2[0::2, 1::2, 1::2, 0::2] = -tba
    T2[1::2, 0::2, 0::2, 1::2] = -tba
    T2[0::2, 0::2, 0::2, 0::2] = t2 - tba
    T2[1::2, 1::2, 1::2, 1::2] = t2 - tba
    T1 = None
    if t1 is not None:
        T1 = np.zeros((2 * o, 2 * v), dtype=complex)
        T1[0::2, 0::2] = t1
        T1[1::2, 1::2] = t1
    return T1, T2


class AATOracle:
    """ov: spin-orbital overlaps keyed like apyib_gb300.aats.AAT.from_overlaps;
    T: dict u / np / nn / mp / mn of [t0, t1, t2] (spin-orbital)."""

    def __init__(self, ov, T, o, f, singles, h, b):
        self.ov, self.T, self.o, self.f, self.singles = ov, T, o, f, singles
        self.pref = 1 / (4 * h * b)

    def _norm(self, T):
        s = T[0] ** 2 + 0.25 * np.sum(np.conjugate(T[2]) * T[2])
        if self.singles:
            s += np.sum(np.conjugate(T[1]) * T[1])
        return 1 / np.sqrt(s)

    def norms(self, a, b, normalization):
        if normalization == "intermediate":
            return 1, 1, 1, 1, 1
        T = self.T
        return (self._norm(T["u"]), self._norm(T["np"][a]), self._norm(T["nn"][a]),
                self._norm(T["mp"][b]), self._norm(T["mn"][b]))

    def term(self, a, b, r, s, normalization):
        """apyib/aats.py:161-517 for the (bra rank r, ket rank s) term."""
        N, N_np, N_nn, N_mp, N_mn = self.norms(a, b, normalization)
        ov, T, o, f = self.ov, self.T, self.o, self.f

        def Q(key, x, y):
            return q(ov[key], o, f, r, x, s, y)

        def four(x, y):
            return (Q(("pp", a, b), x, y) * N_np * N_mp - Q(("pn", a, b), x, y) * N_np * N_mn
                    - Q(("np", a, b), x, y) * N_nn * N_mp + Q(("nn", a, b), x, y) * N_nn * N_mn)
        t = {k: T["u"][k] for k in (1, 2)}
        tc = {k: np.conjugate(T["u"][k]) for k in (1, 2)}
        tdH = {k: T["mp"][b][k] - T["mn"][b][k] for k in (1, 2)}
        tdR = {k: np.conjugate(T["np"][a][k] - T["nn"][a][k]) for k in (1, 2)}
        if r == 0 and s == 0:
            I = four(None, None)
        elif r == 0:
            I = Q(("pu", a), None, tdH[s]) * N_np * N - Q(("nu", a), None, tdH[s]) * N_nn * N + four(None, t[s])
        elif s == 0:
            I = Q(("up", b), tdR[r], None) * N * N_mp - Q(("un", b), tdR[r], None) * N * N_mn + four(tc[r], None)
        else:
            I = (Q("uu", tdR[r], tdH[s]) * N * N
                 + Q(("up", b), tdR[r], t[s]) * N * N_mp - Q(("un", b), tdR[r], t[s]) * N * N_mn
                 + Q(("pu", a), tc[r], tdH[s]) * N_np * N - Q(("nu", a), tc[r], tdH[s]) * N_nn * N
                 + four(tc[r], t[s]))
        return self.pref * np.imag(I)
