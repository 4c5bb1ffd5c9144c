"""Helpers shared by the GPU tests (torch device buffers, seeded inputs)."""
import numpy as np


def to_dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def from_dev(t):
    return t.detach().cpu().numpy()


def rand_spinor(rng, ns, nrhs=1):
    v = rng.normal(size=(nrhs, 2 * ns)) + 1j * rng.normal(size=(nrhs, 2 * ns))
    return v[0] if nrhs == 1 else v


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()
