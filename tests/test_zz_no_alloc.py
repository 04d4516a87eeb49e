"""agb_vec_dots_noalloc: the DIIS Gram-row reduction for callers that cannot
allocate device memory (it keeps its block partial sums in a fixed array
inside the library instead of a caller-provided buffer).

Checked through the C ABI against agb_vec_dots, which takes a caller buffer,
on two calls in a row with different inputs and vector counts, so a result
that depended on what the previous call left in the shared array would show.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from apyib_gb300 import _lib  # noqa: E402


def _vecs(rng, n, ny):
    def r():
        a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        return torch.as_tensor(a).cuda()
    return r(), [r() for _ in range(ny)]


def _dots_with_buffer(n1, n2, x, ys, stream):
    lib = _lib.load()
    ny = len(ys)
    out = torch.zeros(ny, dtype=torch.complex128, device="cuda")
    pb = lib.agb_vec_partials_bytes(ny)
    part = torch.empty(int(pb) // 16 + 1, dtype=torch.complex128, device="cuda")
    arr = (ctypes.c_void_p * ny)(*[y.data_ptr() for y in ys])
    _lib.call("agb_vec_dots", n1, n2, 1.0, 4.0, ctypes.c_void_p(x.data_ptr()), arr, ny,
              ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(part.data_ptr()), ctypes.c_size_t(pb), stream)
    return out


def _dots_noalloc(n1, n2, x, ys, stream):
    ny = len(ys)
    out = torch.zeros(ny, dtype=torch.complex128, device="cuda")
    arr = (ctypes.c_void_p * ny)(*[y.data_ptr() for y in ys])
    _lib.call("agb_vec_dots_noalloc", n1, n2, 1.0, 4.0, ctypes.c_void_p(x.data_ptr()), arr, ny,
              ctypes.c_void_p(out.data_ptr()), stream)
    return out


def test_noalloc_dots_match_buffered_dots_twice():
    torch.cuda.set_device(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    for (n1, n2, ny) in [(1200, 50000, 16), (37, 999, 5)]:
        x, ys = _vecs(rng, n1 + n2, ny)
        ref = _dots_with_buffer(n1, n2, x, ys, stream)
        got = _dots_noalloc(n1, n2, x, ys, stream)
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        np.testing.assert_allclose(g, r, rtol=1e-12, atol=0)
        # and against a host reduction
        xh = x.cpu().numpy()
        host = np.array([np.vdot(y.cpu().numpy()[:n1], xh[:n1]) + 4 * np.vdot(y.cpu().numpy()[n1:], xh[n1:])
                         for y in ys])
        np.testing.assert_allclose(g, host, rtol=1e-11)


def test_noalloc_rejects_more_vectors_than_its_scratch_holds():
    rng = np.random.default_rng(12)
    x, ys = _vecs(rng, 64, 17)
    with pytest.raises(_lib.AGBError) as e:
        _dots_noalloc(0, 64, x, ys, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert e.value.status == _lib.AGB_ERR_ARG
