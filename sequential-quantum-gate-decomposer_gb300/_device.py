"""Device-memory plumbing on top of PyTorch (allocation, streams, host<->device copies).

PyTorch only provides memory and streams here; all arithmetic of the hot path runs in
the engine's own CUDA kernels (libsqg.so).  Every function raises when no CUDA device
is present: the package has no CPU fallback.
"""
import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the target image
    torch = None


class DeviceUnavailable(RuntimeError):
    pass


def require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise DeviceUnavailable("the sequential-quantum-gate-decomposer GB300 engine needs a CUDA device; "
                                "no CPU fallback exists")


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def after_current(stream):
    """Makes `stream` (if given and not the current stream) wait for the work queued so far on
    the current stream, where the inputs of a launch were copied or produced."""
    if stream is not None:
        cur = torch.cuda.current_stream()
        if stream != cur:
            stream.wait_stream(cur)


def ptr(t):
    return int(t.data_ptr()) if t is not None else None


def to_device_complex(a, device="cuda"):
    """complex128 numpy/torch array -> contiguous complex128 CUDA tensor."""
    require_cuda()
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=torch.complex128)
        return t.contiguous()
    arr = np.ascontiguousarray(a)
    if arr.dtype != np.complex128:
        raise TypeError("expected a complex128 array, got %s" % arr.dtype)
    return torch.from_numpy(arr).to(device, non_blocking=False)


def to_device_real(a, device="cuda"):
    require_cuda()
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float64).contiguous()
    arr = np.ascontiguousarray(a, dtype=np.float64)
    return torch.from_numpy(arr).to(device)


class Workspace:
    """Grow-only device scratch buffer, reused across calls of one owner."""

    def __init__(self):
        self._buf = None

    def get(self, nbytes):
        require_cuda()
        nbytes = max(int(nbytes), 256)
        if self._buf is None or self._buf.numel() < nbytes:
            self._buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        return self._buf

    def release(self):
        self._buf = None
