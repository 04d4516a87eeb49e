"""The batched AAT terms (aats.AAT.compute_aat_tensor: every overlap of every element
stacked, the determinant-lemma contractions as broadcast batched products) are plain
tensor algebra.  With the package's device helpers pointed at the CPU they run here, and
they must reproduce the reference's own swapped-determinant sums (apyib/aats.py:120-555
run on seeded overlaps and amplitudes; tests/golden/aat_small.npz) term by term summed,
in full and intermediate normalisation, spin-orbital and spatial."""
import os

import numpy as np
import pytest
import torch

from apyib_gb300 import aats

HERE = os.path.dirname(os.path.abspath(__file__))
SMALL = np.load(os.path.join(HERE, "golden", "aat_small.npz"))
PAIRS = [(0, 0), (1, 2), (2, 1)]
TERMS = ["I_00", "I_0D", "I_D0", "I_DD", "I_0S", "I_S0", "I_SS", "I_SD", "I_DS"]


@pytest.fixture
def on_cpu(monkeypatch):
    def to_cpu(x, dtype=torch.complex128):
        t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(x))
        return t.to(dtype=dtype).resolve_conj().contiguous()
    def bmm(A, B, transA=False, conjA=False, transB=False, conjB=False, alpha=1.0):
        A = A.mT if transA else A
        B = B.mT if transB else B
        return alpha * ((A.conj() if conjA else A) @ (B.conj() if conjB else B))

    def bdet_inv(S):
        return torch.linalg.det(S), torch.linalg.inv(S)

    monkeypatch.setattr(aats, "device", lambda: torch.device("cpu"))
    monkeypatch.setattr(aats, "to_dev", to_cpu)
    monkeypatch.setattr(aats, "bmm", bmm)
    monkeypatch.setattr(aats, "bdot", lambda X, Y: (X.reshape(X.shape[0], -1) * Y.reshape(Y.shape[0], -1)).sum(-1))
    monkeypatch.setattr(aats, "bdet_inv", bdet_inv)


def so_overlap(M):
    n = M.shape[0]
    S = np.zeros((2 * n, 2 * n), dtype=complex)
    S[0::2, 0::2] = M
    S[1::2, 1::2] = M
    return S


def small_case(tag, method):
    ov = {}
    for k in SMALL.files:
        if k.startswith(tag + "_ov_"):
            parts = k[len(tag) + 4:].split("_")
            key = parts[0] if len(parts) == 1 else (parts[0],) + tuple(int(p) for p in parts[1:])
            ov[key] = so_overlap(SMALL[k])

    def amps(name):
        return [1.0, SMALL[f"{tag}_T_{name}_1"], SMALL[f"{tag}_T_{name}_2"]]
    T = {k: [amps(f"{k}{i}") for i in range(3)] for k in ("np", "nn", "mp", "mn")}
    return aats.AAT.from_overlaps({"method": method}, ndocc=2, nbf=4, nfzc=0, natom=1, overlaps=ov,
                                  unperturbed_T=amps("u"), nuc_pos_T=T["np"], nuc_neg_T=T["nn"],
                                  mag_pos_T=T["mp"], mag_neg_T=T["mn"], nuc_pert_strength=1e-4,
                                  mag_pert_strength=1e-4)


@pytest.mark.parametrize("norm", ["full", "intermediate"])
def test_batched_terms_match_reference_determinant_sums(on_cpu, norm):
    full = small_case("so", "CISD_SO").compute_aat_tensor(norm)
    for a, b in PAIRS:
        ref = sum(float(SMALL[f"so_{norm}_{a}_{b}_{name}"]) for name in TERMS)
        assert abs(full[a, b] - ref) <= 1e-9 * max(1.0, abs(ref)), (a, b, full[a, b], ref)
    sp = small_case("sp", "CISD").compute_aat_tensor("intermediate")
    for a, b in PAIRS:
        ref = float(SMALL[f"sp_intermediate_{a}_{b}_total"])
        assert abs(sp[a, b] - ref) <= 1e-9 * max(1.0, abs(ref)), (a, b, sp[a, b], ref)
