"""Fixed-order reductions (replaces the reference's dsplat/kernels/reduce.py)."""

from __future__ import annotations

import torch

from . import _lib
from ._lib import call, ptr, real_view


def energy(value, reference):
    """sum |value - reference|^2 of two complex tensors, accumulated in float64.

    Returns a 0-d float64 tensor on the device; the sum order is fixed, so equal
    inputs give bitwise equal results.
    """
    v = real_view(value).reshape(-1, 2)
    r = real_view(reference).reshape(-1, 2)
    out = torch.empty((), dtype=torch.float64, device=v.device)
    nbytes = _lib.query("dsg_energy_workspace_bytes", len(v))
    work, nbytes = _lib.workspace(nbytes, v.device)
    call("dsg_energy", ptr(v), ptr(r), len(v), ptr(out), ptr(work), nbytes, _lib.stream(v.device))
    return out
