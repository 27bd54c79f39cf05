"""Float64 range response of the row-basis SVD (replaces the reference's
dsplat/kernels/response.py)."""

from __future__ import annotations

import torch

from . import _lib
from ._lib import call, ptr


def range_response(config, low, high, count, device):
    """Float64 responses [bins, count] of count peak positions spread over [low, high]."""
    out = torch.empty(
        (config.num_range_bins, count, 2), device=device, dtype=torch.float64
    )
    call(
        "dsg_range_response", float(low), float(high), int(count), config.num_range_bins,
        config.adc_samples, config.n_fft, ptr(out), _lib.stream(out.device),
    )  # fmt: skip
    return torch.view_as_complex(out)
