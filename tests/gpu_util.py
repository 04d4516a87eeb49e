"""Shared helpers for the GPU tests."""
import glob
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_gold(name):
    return dict(np.load(os.path.join(GOLD, name)))


def so_golden_files(with_inputs=False):
    files = sorted(glob.glob(os.path.join(GOLD, "so_*.npz")))
    if with_inputs:
        files = [f for f in files if "B" in np.load(f).files]
    return files


def crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
