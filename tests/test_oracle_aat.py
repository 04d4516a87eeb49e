"""The AAT oracle (oracle/aats.py: the reference's swapped-row/column determinant
sums restated, batched) against the reference's own apyib/aats.py term methods
run on the same seeded overlaps and amplitudes (tests/golden/make_golden_aat.py
-> aat_small.npz): all nine spin-orbital CISD terms in full and intermediate
normalisation, and the spatial-orbital CISD total (the same sums over the
spin-orbital expansion of the closed-shell amplitudes) in intermediate
normalisation.  In full normalisation the reference's spatial routine
(apyib/aats.py:653-700) scales the amplitudes before differencing them while
its spin-orbital routine (:134-158) scales the determinant terms; the
reference's own golden arrays for spatial and spin-orbital MP2
(apyib/tests/test_011_AAT.py, test_012_AAT_SO.py) are identical, and the
spin-orbital definition is the one followed here for both."""
import os

import numpy as np
import pytest

from oracle.aats import AATOracle, so_amplitudes

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "aat_small.npz"))
PAIRS = [(0, 0), (1, 2), (2, 1)]
TERMS = {"I_00": (0, 0), "I_0D": (0, 2), "I_D0": (2, 0), "I_DD": (2, 2), "I_0S": (0, 1), "I_S0": (1, 0),
         "I_SS": (1, 1), "I_SD": (1, 2), "I_DS": (2, 1)}


def so_overlap(M):
    n = M.shape[0]
    S = np.zeros((2 * n, 2 * n), dtype=complex)
    S[0::2, 0::2] = M
    S[1::2, 1::2] = M
    return S


def load(tag, spatial):
    ov = {}
    for k in G.files:
        if k.startswith(tag + "_ov_"):
            parts = k[len(tag) + 4:].split("_")
            key = parts[0] if len(parts) == 1 else (parts[0],) + tuple(int(p) for p in parts[1:])
            ov[key] = so_overlap(G[k])

    def amps(name):
        t1, t2 = G[f"{tag}_T_{name}_1"], G[f"{tag}_T_{name}_2"]
        if spatial:
            t1, t2 = so_amplitudes(t1, t2)
        return [1.0, t1, t2]
    T = {"u": amps("u")}
    for key, n in (("np", 3), ("nn", 3), ("mp", 3), ("mn", 3)):
        T[key] = [amps(f"{key}{i}") for i in range(n)]
    return ov, T


@pytest.mark.parametrize("norm", ["full", "intermediate"])
def test_spin_orbital_terms_match_reference(norm):
    ov, T = load("so", False)
    orc = AATOracle(ov, T, o=4, f=0, singles=True, h=1e-4, b=1e-4)
    for a, b in PAIRS:
        for name, (r, s) in TERMS.items():
            ref = float(G[f"so_{norm}_{a}_{b}_{name}"])
            got = orc.term(a, b, r, s, norm)
            assert abs(got - ref) <= 1e-9 * max(1.0, abs(ref)), (norm, a, b, name, got, ref)


@pytest.mark.parametrize("norm", ["intermediate"])
def test_spatial_total_matches_reference(norm):
    ov, T = load("sp", True)
    orc = AATOracle(ov, T, o=4, f=0, singles=True, h=1e-4, b=1e-4)
    for a, b in PAIRS:
        ref = float(G[f"sp_{norm}_{a}_{b}_total"])
        got = sum(orc.term(a, b, r, s, norm) for r, s in TERMS.values())
        assert abs(got - ref) <= 1e-9 * max(1.0, abs(ref)), (norm, a, b, got, ref)
