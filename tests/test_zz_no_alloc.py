"""dsg_surfel_vjp_fixed_scratch: the VJP for callers that cannot allocate device memory.

Collected last (file name) so that it also runs after every other test has used the
library in the same process; it must pass alone in a fresh process as well. Both entry
points are called through the C ABI; the fixed-scratch variant must agree with
dsg_surfel_vjp (which takes a caller workspace) on consecutive calls that share the
library's one scratch array.
"""

from __future__ import annotations

import ctypes

import pytest
import torch

from conftest import aperture_grid, rel_l2, surfels

DERIV_TOL = 1e-4


def _inputs(config, side, count, seed):
    positions = aperture_grid(side)
    params = surfels(count, seed=seed)
    generator = torch.Generator().manual_seed(seed + 100)
    weights = torch.complex(torch.rand(count, generator=generator) + 0.5,
                            torch.randn(count, generator=generator) * 0.2)  # fmt: skip
    upstream = torch.complex(torch.randn(len(positions), config.num_range_bins, generator=generator),
                             torch.randn(len(positions), config.num_range_bins, generator=generator))  # fmt: skip
    return positions, params["centers"], params["normals"], weights.cuda(), upstream.cuda()


def _gradients(name, config, positions, centers, normals, weights, upstream):
    from dsplat.kernels import _lib

    chirp = _lib.chirp(config, 0.0)
    count, apertures = len(centers), len(positions)
    w, u = torch.view_as_real(weights).contiguous(), torch.view_as_real(upstream).contiguous()
    gc = torch.full((count, 3), float("nan"), device="cuda")
    gn = torch.full((count, 3), float("nan"), device="cuda")
    gw = torch.full((count, 2), float("nan"), device="cuda")
    stream = _lib.stream(centers.device)
    args = (_lib.ptr(positions), apertures, _lib.ptr(centers), _lib.ptr(normals), _lib.ptr(w), count,
            _lib.ptr(u), _lib.ptr(gc), _lib.ptr(gn), _lib.ptr(gw))  # fmt: skip
    if name == "dsg_surfel_vjp":
        nbytes = _lib.query("dsg_surfel_reduce_workspace_bytes", chirp, apertures, count, 8)
        work, nbytes = _lib.workspace(nbytes, centers.device)
        _lib.call(name, chirp, *args, _lib.ptr(work), nbytes, stream)
    else:
        _lib.call(name, chirp, *args, stream)
    return gc, gn, torch.view_as_complex(gw)


@pytest.mark.gpu
def test_fixed_scratch_vjp_matches_workspace_vjp_on_consecutive_calls():
    from dsplat import FMCWConfig

    config = FMCWConfig()
    # Two differently sized problems in a row: the second call reuses the scratch that the
    # first left behind, with a different number of aperture chunks per surfel.
    for side, count, seed in ((32, 300, 1), (16, 700, 2)):
        inputs = _inputs(config, side, count, seed)
        fixed = _gradients("dsg_surfel_vjp_fixed_scratch", config, *inputs)
        expected = _gradients("dsg_surfel_vjp", config, *inputs)
        torch.cuda.synchronize()
        for a, e in zip(fixed, expected):
            assert torch.isfinite(torch.view_as_real(a) if a.is_complex() else a).all()
            assert rel_l2(a, e) < DERIV_TOL


def test_fixed_scratch_vjp_rejects_sizes_beyond_its_scratch():
    """The size check runs on the host before any device call, so it needs no GPU."""
    from dsplat import FMCWConfig
    from dsplat.kernels import _lib

    lib = _lib.library()
    chirp = _lib.chirp(FMCWConfig())
    limit = 4 << 20
    surfels_over = limit // 32 + 16  # one aperture chunk of 8 floats per surfel
    assert lib.dsg_surfel_reduce_workspace_bytes(ctypes.byref(chirp), 64, surfels_over, 8) > limit
    dummy = ctypes.c_void_p(256)  # never dereferenced: the call returns before using it
    status = lib.dsg_surfel_vjp_fixed_scratch(ctypes.byref(chirp), dummy, 64, dummy, dummy, dummy,
                                              surfels_over, dummy, dummy, dummy, dummy, None)  # fmt: skip
    assert status == 3 and lib.dsg_error_string(status) == b"workspace missing or too small"
