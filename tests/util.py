"""numpy <-> torch helpers for the tests."""
import numpy as np
import torch

NP_TO_TORCH = {np.dtype(np.uint8): torch.uint8, np.dtype(np.int8): torch.int8,
               np.dtype(np.uint32): torch.uint32, np.dtype(np.int32): torch.int32,
               np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}
TORCH_TO_NP = {v: k for k, v in NP_TO_TORCH.items()}


def to_dev(a: np.ndarray, device="cuda") -> torch.Tensor:
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        return torch.from_numpy(a.view(np.int32)).to(device).view(torch.uint32)
    return torch.from_numpy(a).to(device)


def to_np(t: torch.Tensor) -> np.ndarray:
    if t.dtype == torch.uint32:
        return t.view(torch.int32).cpu().numpy().view(np.uint32)
    return t.cpu().numpy()


def empty_pitched(h: int, w: int, pitch: int, dtype, device="cuda", fill=None) -> torch.Tensor:
    """A (h, w) view with row stride `pitch` elements into a larger buffer."""
    base_dtype = torch.int32 if dtype == torch.uint32 else dtype
    base = torch.empty(h * pitch, dtype=base_dtype, device=device)
    if fill is not None:
        base.fill_(fill)
    if dtype == torch.uint32:
        base = base.view(torch.uint32)
    return base.as_strided((h, w), (pitch, 1))


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a).view(np.uint8)
