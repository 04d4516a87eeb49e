"""The decomposition the (l, s)-symmetric J/K kernels use (jk_sym_kernel, jk_sym64_kernel in
apyib_gb300/csrc/misc.cu), restated in NumPy and checked against the oracle's full-tensor
J/K (apyib/hf_wfn.py:81, apyib/utils.py:249): with e[m][x][y][z] = (mx|yz) symmetric in
(y, z), reading only z >= y,
    J[m][x] = sum_{y<=z} e S[y][z],  S = D + D^T off the diagonal, S[y][y] = D[y][y],
    K[m][y] += sum_{x, z>=y} e D[x][z],  K[m][z] += sum_{x, y<z} e D[x][y],
for a complex, non-Hermitian D."""
import numpy as np

from oracle import port


def jk_symmetric_half(h, eri, D, scale):
    n = D.shape[0]
    S = D + D.T
    S[np.diag_indices(n)] = np.diag(D)
    J = np.zeros((n, n), dtype=complex)
    K = np.zeros((n, n), dtype=complex)
    for y in range(n):
        z = np.arange(y, n)
        e = eri[:, :, y, y:]                                  # [m, x, z >= y]
        J += np.einsum("mxz,z->mx", e, S[y, y:])
        K[:, y] += np.einsum("mxz,xz->m", e, D[:, y:])
        off = z > y
        K[:, z[off]] += np.einsum("mxz,x->mz", e[:, :, off], D[:, y])
    return h + scale * (2 * J - K)


def test_symmetric_half_decomposition_matches_full_jk():
    rng = np.random.default_rng(11)
    for n in (1, 2, 5, 9):
        A = rng.standard_normal((6, n, n))
        A = A + A.transpose(0, 2, 1)
        eri = np.einsum("Lmn,Lls->mnls", A, A)
        eri = 0.5 * (eri + eri.transpose(0, 1, 3, 2))
        D = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))      # not Hermitian
        h = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        got = jk_symmetric_half(h, eri, D, 0.5)
        ref = port.jk_fock(h, eri, D, 0.5)
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), n
