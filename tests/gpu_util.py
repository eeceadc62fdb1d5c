"""Helpers for the GPU parity tests: device grids held in torch tensors (plain
device memory) and readable first-difference reports."""
import numpy as np


def to_device(torch, g: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(g)).cuda()


def stream_ptr(torch) -> int:
    return torch.cuda.current_stream().cuda_stream


def describe_diff(got: np.ndarray, exp: np.ndarray, step) -> str:
    Y, Z, X = exp.shape
    d = np.flatnonzero(got.reshape(-1) != exp.reshape(-1))
    if d.size == 0:
        return "grids equal"
    i = int(d[0])
    x, z, y = i % X, (i // X) % Z, i // (X * Z)
    return (f"step {step}: {d.size} cells differ; first idx {i} (x={x}, y={y}, z={z}) "
            f"got {got.reshape(-1)[i]} expected {exp.reshape(-1)[i]}")
