"""Device-buffer plumbing between torch tensors and the C ABI.

Particle records are float32 float4 rows: xm = {x, y, z, m}, vel = {vx, vy,
vz, 0}, acc = {ax, ay, az, 0}.  torch only provides the memory and the
stream; all arithmetic runs in the CUDA library.
"""
from __future__ import annotations

import numpy as np
import torch


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 gravity engine needs a CUDA device; none is visible")
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda":
        raise ValueError(f"device must be a CUDA device, got {dev}")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def stream_handle(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor, name: str = "tensor", dtype=torch.float32, rows4: bool = True) -> int:
    """Raw device pointer of a contiguous CUDA tensor (checked)."""
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must live on a CUDA device")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if rows4 and (t.dim() != 2 or t.shape[1] != 4):
        raise ValueError(f"{name} must have shape (n, 4), got {tuple(t.shape)}")
    return t.data_ptr()


def pack_xm(pos, mass, device) -> torch.Tensor:
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    mass = np.asarray(mass, dtype=np.float64).reshape(-1)
    host = np.empty((pos.shape[0], 4), np.float32)
    host[:, :3] = pos
    host[:, 3] = mass
    return torch.from_numpy(host).to(device)


def pack_vec(v, device) -> torch.Tensor:
    v = np.asarray(v, dtype=np.float64).reshape(-1, 3)
    host = np.zeros((v.shape[0], 4), np.float32)
    host[:, :3] = v
    return torch.from_numpy(host).to(device)


def empty4(n: int, device) -> torch.Tensor:
    return torch.zeros((n, 4), dtype=torch.float32, device=device)


class FieldView:
    """Reference-style field access (``to_numpy`` / ``from_numpy``) over a
    column slice of a float4 device buffer; ``on_write`` (optional) is
    called after every write through the view."""

    def __init__(self, buf: torch.Tensor, cols, on_write=None):
        self._buf = buf
        self._cols = cols
        self._on_write = on_write

    def _written(self) -> None:
        if self._on_write is not None:
            self._on_write()

    @property
    def tensor(self) -> torch.Tensor:
        return self._buf[:, self._cols]

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    def to_numpy(self) -> np.ndarray:
        return self.tensor.detach().to("cpu", torch.float64).numpy()

    def from_numpy(self, arr) -> None:
        src = torch.as_tensor(np.asarray(arr, dtype=np.float32)).reshape(self.shape)
        self._buf[:, self._cols] = src.to(self._buf.device)
        self._written()

    def __array__(self, dtype=None, copy=None):
        a = self.to_numpy()
        return a.astype(dtype) if dtype is not None else a


def field_values(x, device) -> torch.Tensor:
    """float32 device tensor of a reference-style field (anything with
    ``to_numpy``), a FieldView, a numpy array or a torch tensor."""
    if isinstance(x, FieldView):
        t = x.tensor
    elif isinstance(x, torch.Tensor):
        t = x
    elif hasattr(x, "to_numpy"):
        t = torch.from_numpy(np.ascontiguousarray(x.to_numpy()))
    else:
        t = torch.as_tensor(np.asarray(x))
    return t.to(device=device, dtype=torch.float32)


def write_rows(dst, values: torch.Tensor) -> None:
    """Write values (device, rows 0..len-1) into the first rows of dst: a
    FieldView, a torch tensor, a numpy array or a reference-style field
    (``to_numpy`` / ``from_numpy``)."""
    n = values.shape[0]
    if isinstance(dst, FieldView):
        dst._buf[:n, dst._cols] = values.to(dst._buf.dtype)
        dst._written()
    elif isinstance(dst, torch.Tensor):
        dst[:n] = values.to(device=dst.device, dtype=dst.dtype)
    elif isinstance(dst, np.ndarray):
        dst[:n] = values.double().cpu().numpy().reshape(dst[:n].shape)
    else:
        full = np.array(dst.to_numpy())
        full[:n] = values.double().cpu().numpy().reshape(full[:n].shape)
        dst.from_numpy(full)


def pick_device(*xs) -> torch.device:
    """The CUDA device of the first CUDA tensor (or FieldView) among xs,
    else the current CUDA device."""
    for x in xs:
        if isinstance(x, FieldView):
            return x.tensor.device
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    return require_cuda()
