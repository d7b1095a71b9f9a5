"""Device plumbing shared by the host modules: tensors, streams, pointers.

PyTorch provides device memory and streams; all compute goes through the
C-ABI library (``_lib``).  Nothing here computes on the CPU."""

import numpy as np
import torch

from . import _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("mahakala_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU fallback")
    _lib.load()


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def f64(x, dev=None):
    """Contiguous float64 CUDA tensor view/copy of an array-like."""
    dev = dev or device()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def ptr(t):
    return None if t is None else t.data_ptr()


def to_numpy(t):
    return t.detach().cpu().numpy()
