"""Device buffers and streams.

PyTorch is used only as the allocator (caching CUDA memory) and for the
current CUDA stream; every computation on rays is a kernel of
libbatoid_gb300.so.
"""
import numpy as np
import torch

_DEV = None


def device():
    global _DEV
    if _DEV is None:
        if not torch.cuda.is_available():
            raise RuntimeError("batoid_gb300 needs a CUDA device (no CPU fallback)")
        _DEV = torch.device("cuda", torch.cuda.current_device())
    return _DEV


def stream_ptr():
    """cudaStream_t of torch's current stream, as an int for ctypes."""
    return torch.cuda.current_stream(device()).cuda_stream


def empty(shape, dtype=torch.float64):
    return torch.empty(shape, dtype=dtype, device=device())


def to_device(a, dtype=torch.float64):
    """numpy / scalar / tensor -> contiguous device tensor (copy)."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device(), dtype=dtype).contiguous()
    npdt = np.float64 if dtype == torch.float64 else np.uint8
    arr = np.ascontiguousarray(np.asarray(a, dtype=npdt))
    return torch.from_numpy(arr).to(device())


def to_host(t):
    return t.detach().cpu().numpy()


def ptr(t):
    return t.data_ptr() if t is not None and t.numel() > 0 else None
