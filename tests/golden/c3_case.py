"""Inputs and probe layout of the o/v = 40/160 residual fixture (c3res_40_160.npz),
shared by its generator (make_golden_c3.py, which runs the reference) and the GPU test
(which must not load the reference)."""
import hashlib

import numpy as np

O, V, SEED = 40, 160, 21
NPROBE = 4096
FIXTURE = f"c3res_{O}_{V}.npz"


def digest(*arrs):
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def probe_indices(o, v, n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, o, n), rng.integers(0, o, n), rng.integers(0, v, n), rng.integers(0, v, n)])


def projection_weights(o, v, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((o, o, v, v))


def perturbed_fock(prob, o, v, seed):
    """F_SO plus a spin-conserving Hermitian perturbation (every Fock term counts)."""
    F = prob.fock_so()
    rng = np.random.default_rng(seed + 1000)
    pert = (rng.standard_normal(F.shape) + 1j * rng.standard_normal(F.shape)) * 0.01
    pert = pert + pert.conj().T
    mask = np.add.outer(np.arange(o + v) % 2, np.arange(o + v) % 2) % 2 == 0
    return F + pert * mask
