"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

GUARD = 64  # guard words around every output buffer


def guarded(n, bits, kind):
    """Output tensor with GUARD canary words on each side; returns (full, view)."""
    if bits == 32:
        dt = torch.int32 if kind == 0 else torch.float32
    else:
        dt = torch.int64 if kind == 0 else torch.float64
    full = torch.empty(n + 2 * GUARD, dtype=dt, device="cuda")
    full.view(torch.int32 if bits == 32 else torch.int64).fill_(-0x5A5A5A5A)
    return full, full[GUARD:GUARD + n]


def check_guards(full, bits):
    v = full.view(torch.int32 if bits == 32 else torch.int64).cpu().numpy()
    assert (v[:GUARD] == -0x5A5A5A5A).all(), "write before the output buffer"
    assert (v[-GUARD:] == -0x5A5A5A5A).all(), "write after the output buffer"


def as_np_bits(t, bits):
    """Raw bits of a CUDA tensor as a numpy unsigned array."""
    a = t.cpu().numpy()
    return a.view(np.uint32 if bits == 32 else np.uint64)


def np_bits(a, bits):
    return np.ascontiguousarray(a).view(np.uint32 if bits == 32 else np.uint64)
