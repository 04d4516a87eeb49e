"""Device helpers: CUDA tensors, raw pointers and the current stream.

The product path needs a CUDA device and the in-tree library; both are
checked here and a missing one raises (there is no CPU fallback)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("apyib_gb300 needs a CUDA GPU (GB300, sm_103a); none is available")
    _lib.load()


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    """Raw device pointer of a tensor whose storage holds exactly its values
    (torch's lazy conjugate / negative views do not, and are refused)."""
    if t is None:
        return ctypes.c_void_p(0)
    if t.is_conj() or t.is_neg():
        raise ValueError("lazy conj/neg view passed to the C ABI; call resolve_conj()/resolve_neg() first")
    return ctypes.c_void_p(t.data_ptr())


def materialize(t):
    """Contiguous tensor with any lazy conjugation or negation applied."""
    return t.resolve_conj().resolve_neg().contiguous()


def to_dev(x, dtype=torch.complex128):
    """NumPy array or tensor -> contiguous CUDA tensor of ``dtype``."""
    dev = device()
    if isinstance(x, torch.Tensor):
        return materialize(x.to(device=dev, dtype=dtype))
    return torch.as_tensor(np.ascontiguousarray(x)).to(device=dev, dtype=dtype).contiguous()


def to_host(t):
    return t.detach().cpu().numpy()


def empty(n, dtype=torch.complex128):
    return torch.empty(n, dtype=dtype, device=device())


def workspace(nbytes):
    """A 256-byte aligned device buffer (torch's caching allocator)."""
    buf = torch.empty(max(int(nbytes), 256) + 256, dtype=torch.uint8, device=device())
    off = (-buf.data_ptr()) % 256
    return buf, buf.data_ptr() + off, int(nbytes)
