"""Separable Dirichlet atoms on a spectral grid, in bin units (replaces the reference's
dsplat/kernels/spectral.py bindings of spectral.slang with libdsplat_gb300.so calls)."""

from __future__ import annotations

import torch
from torch.autograd.function import once_differentiable

from . import _lib
from ._lib import call, f32, ptr, real_view

WINDOWS = ("rect", "hann", "hamming", "kaiser")


def _grid(grid, device):
    """C struct of a SpectralGrid and its Kaiser taps [dim, max taps] (sum-normalized)."""
    dim = len(grid.shape)
    width = max(grid.samples)
    taps = torch.zeros((dim, width), dtype=torch.float32, device=device)
    if grid.window == "kaiser":
        for d, n in enumerate(grid.samples):
            w = torch.kaiser_window(n, periodic=False, beta=grid.beta, dtype=torch.float64)
            taps[d, :n] = (w / w.sum()).to(device, torch.float32)
    c = _lib.Grid()
    c.dim = dim
    for d in range(3):
        c.nfft[d] = grid.shape[d] if d < dim else 1
        c.samples[d] = grid.samples[d] if d < dim else 1
    c.window = WINDOWS.index(grid.window)
    c.max_taps = width
    c.radius = float(grid.radius)
    return c, taps.contiguous()


def design(grid, centers, bins, derivatives=False):
    """Dictionary A [M, S] and, with derivatives, dA/dcenters [M, S, D]."""
    centers, bins = f32(centers), f32(bins)
    c, taps = _grid(grid, centers.device)
    a = torch.empty((len(bins), len(centers), 2), dtype=torch.float32, device=centers.device)
    da = (
        torch.empty((len(bins), len(centers), centers.shape[1], 2), dtype=torch.float32,
                    device=centers.device)
        if derivatives else None
    )  # fmt: skip
    call(
        "dsg_spectral_design", c, ptr(taps), ptr(centers), len(centers), ptr(bins), len(bins),
        ptr(a), ptr(da), _lib.stream(centers.device),
    )  # fmt: skip
    a = torch.view_as_complex(a)
    return (a, torch.view_as_complex(da)) if derivatives else a


def _forward(grid, centers, coeff, bins):
    centers, bins = f32(centers), f32(bins)
    c, taps = _grid(grid, centers.device)
    out = torch.empty((len(bins), 2), dtype=torch.float32, device=centers.device)
    call(
        "dsg_spectral_render", c, ptr(taps), ptr(centers), len(centers), ptr(coeff.contiguous()),
        ptr(bins), len(bins), ptr(out), _lib.stream(centers.device),
    )  # fmt: skip
    return out


def _backward(grid, centers, coeff, bins, upstream):
    centers, bins = f32(centers), f32(bins)
    c, taps = _grid(grid, centers.device)
    gc = torch.empty_like(centers)
    gb = torch.empty((len(centers), 2), dtype=torch.float32, device=centers.device)
    nbytes = _lib.query("dsg_spectral_vjp_workspace_bytes", c, len(centers), len(bins))
    work, nbytes = _lib.workspace(nbytes, centers.device)
    call(
        "dsg_spectral_vjp", c, ptr(taps), ptr(centers), len(centers), ptr(coeff.contiguous()),
        ptr(upstream.contiguous()), ptr(bins), len(bins), ptr(gc), ptr(gb), ptr(work), nbytes,
        _lib.stream(centers.device),
    )  # fmt: skip
    return gc, gb


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, centers, coeff, grid, bins):
        ctx.save_for_backward(centers, coeff, bins)
        ctx.grid = grid
        return _forward(grid, centers, coeff, bins)

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        centers, coeff, bins = ctx.saved_tensors
        gc, gb = _backward(ctx.grid, centers, coeff, bins, grad.contiguous())
        return gc.to(centers.dtype), gb, None, None  # the kernel works in float32


def render(grid, centers, coefficients, bins):
    """Coherent sum of complex atoms at the given bins; differentiable in both inputs."""
    output = _Render.apply(centers.contiguous(), real_view(coefficients), grid, bins)
    return torch.view_as_complex(output)


def jvp(grid, centers, coefficients, delta_centers, delta_coefficients, bins):
    centers, bins, dc = f32(centers), f32(bins), f32(delta_centers)
    c, taps = _grid(grid, centers.device)
    out = torch.empty((len(bins), 2), dtype=torch.float32, device=centers.device)
    call(
        "dsg_spectral_jvp", c, ptr(taps), ptr(centers), len(centers),
        ptr(real_view(coefficients)), ptr(dc), ptr(real_view(delta_coefficients)), ptr(bins),
        len(bins), ptr(out), _lib.stream(centers.device),
    )  # fmt: skip
    return torch.view_as_complex(out)


def vjp(grid, centers, coefficients, upstream, bins):
    """Gradients of Re(conj(upstream) . render) for centers and complex coefficients."""
    gc, gb = _backward(grid, centers, real_view(coefficients), bins, real_view(upstream))
    return gc, torch.view_as_complex(gb)
