"""Host-side logic that needs no GPU: the content key of the cross-geometry AO overlap
cache and the exact (l, s)-symmetry test that picks the J/K kernel."""
import numpy as np
import torch

from apyib_gb300 import basis as B
from apyib_gb300.linalg import last_pair_symmetric
from apyib_gb300.utils import _basis_fingerprint

WATER = """
O 0.0  0.0     {z}
H 0.0  0.7572 -0.4692
H 0.0 -0.7572 -0.4692
units angstrom
no_com
no_reorient
symmetry c1
"""


def _basis(z=0.1173, name="cc-pVDZ", puream=None):
    return B.BasisSet.build(B.parse_geometry(WATER.format(z=z)), name, puream=puream)


def test_overlap_cache_key_follows_basis_content():
    """Equal contents give one key whatever the object; a moved nucleus, another basis or
    a Cartesian instead of a pure set gives another."""
    k = _basis_fingerprint(_basis())
    assert k == _basis_fingerprint(_basis())
    assert k != _basis_fingerprint(_basis(z=0.1173 + 1e-9))
    assert k != _basis_fingerprint(_basis(name="6-31G"))
    assert k != _basis_fingerprint(_basis(puream=False))
    assert _basis_fingerprint(object()) is None          # no shell arrays: never cached


def test_last_pair_symmetry_check_and_its_cache():
    rng = np.random.default_rng(0)
    a = torch.as_tensor(rng.standard_normal((3, 4, 5, 5)))
    sym = 0.5 * (a + a.transpose(2, 3))
    assert last_pair_symmetric(sym)
    assert last_pair_symmetric(sym)                      # cached verdict, same answer
    sym[0, 1, 2, 3] += 1.0                               # in place: the version changes, checked again
    assert not last_pair_symmetric(sym)
    assert not last_pair_symmetric(a)
    assert last_pair_symmetric(torch.zeros((2, 2, 3, 3), dtype=torch.float64))
