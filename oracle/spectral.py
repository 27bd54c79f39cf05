"""Float64 separable spectral atoms (oracle; test-only). Restates
tests/reference/oracle.py:10-31 (spectral_design) with render, JVP and VJP on top."""

from __future__ import annotations

import torch

from .kernel import windowed


def design(grid, centers, bins):
    """Dictionary [M, S] and its center derivative [M, S, D] in complex128."""
    centers, bins = centers.double().cpu(), bins.double().cpu()
    parts = []
    for d, (n, f) in enumerate(zip(grid.samples, grid.shape, strict=True)):
        delta = bins[:, None, d] - centers[None, :, d]
        k, dk = windowed(delta, n, f, grid.window, grid.beta)
        if grid.radius:
            inside = (delta - f * torch.round(delta / f)).abs() <= grid.radius
            k, dk = k * inside, dk * inside
        parts.append((k, dk))
    a = torch.ones((len(bins), len(centers)), dtype=torch.complex128)
    for k, _ in parts:
        a = a * k
    derivatives = []
    for d, (_, dk) in enumerate(parts):
        value = -dk
        for other, (k, _) in enumerate(parts):
            if other != d:
                value = value * k
        derivatives.append(value)
    return a, torch.stack(derivatives, -1)


def render(grid, centers, coefficients, bins):
    a, _ = design(grid, centers, bins)
    return a @ coefficients.cpu().to(torch.complex128)


def jvp(grid, centers, coefficients, delta_centers, delta_coefficients, bins):
    a, da = design(grid, centers, bins)
    b = coefficients.cpu().to(torch.complex128)
    return (da * delta_centers.cpu().double()[None]).sum(-1) @ b + a @ delta_coefficients.cpu().to(torch.complex128)


def vjp(grid, centers, coefficients, upstream, bins):
    a, da = design(grid, centers, bins)
    b = coefficients.cpu().to(torch.complex128)
    u = upstream.cpu().to(torch.complex128)
    gc = (u.conj()[:, None, None] * da * b[None, :, None]).real.sum(0)
    gb = (a.conj() * u[:, None]).sum(0)
    return gc, gb
