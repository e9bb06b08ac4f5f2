"""Shared helpers for the GPU parity tests (calls go through the C ABI)."""
import numpy as np
import torch

from rocket_gb300.kernels import CompositionVectorKernels

NSYM = {"protein": 21, "DNA": 4}


def to_device_bytes(seq: bytes) -> torch.Tensor:
    if len(seq) == 0:
        return torch.empty(1, dtype=torch.uint8, device="cuda")
    return torch.frombuffer(bytearray(seq), dtype=torch.uint8).to("cuda")


def build_gpu(seq: bytes, k: int, alphabet: str = "protein", max_size: int = None):
    """buildCompositionVector through CompositionVectorKernels (JNA-style call)."""
    if max_size is None:
        max_size = min(NSYM[alphabet] ** k, 21 * len(seq) + 64)
    ker = CompositionVectorKernels(alphabet, k, max_size, len(seq))
    d_in = to_device_bytes(seq)
    keys = torch.empty(max_size, dtype=torch.int32, device="cuda")
    vals = torch.empty(max_size, dtype=torch.float32, device="cuda")
    n = ker.build_vector_gpu(d_in, keys, vals, len(seq))
    return n, keys.cpu().numpy().view(np.uint32), vals.cpu().numpy()


def ulp_diff(a: np.ndarray, b: np.ndarray) -> int:
    """Max distance in float32 ulps (NaN == NaN)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if len(a) == 0:
        return 0
    both_nan = np.isnan(a) & np.isnan(b)
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    d = np.abs(ia - ib)
    d[both_nan] = 0
    d[np.isnan(a) ^ np.isnan(b)] = 1 << 40
    return int(d.max())
