"""CPU float64 VarPro refit of the oracle: the reference arm and CPU baseline of bench.py.

One full-data refit is what every DSFW step does at least twice (the merged
replacement's accepted support and the joint Gauss-Newton proposal are each refitted
on all observations; reference: dsplat/varpro.py:139-144, dsplat/replacement.py:259-267,
dsplat/refinement.py:490-494). This module runs that refit with the reference's
arithmetic restated in float64 PyTorch on the host cores: dictionary columns from the
closed form, projection onto the row basis of the range response (float64 SVD),
normal equations, Cholesky solve, and the rendered objective. Test infrastructure:
it never runs inside the product path.
"""

from __future__ import annotations

import time

import torch

from . import fmcw as ofmcw

DTYPE = torch.float64


def row_basis(config, positions, lower, upper):
    """Shared row basis U^H [rank, K] (complex128) of every peak position inside the box."""
    lo = torch.as_tensor(lower, dtype=DTYPE)
    hi = torch.as_tensor(upper, dtype=DTYPE)
    pos = positions.double()
    nearest = torch.minimum(torch.maximum(pos, lo), hi)
    farthest = torch.where((pos - lo).abs() > (pos - hi).abs(), lo, hi)
    spacing = config.range_bin_spacing_m
    low = float(((pos - nearest).norm(dim=1) / spacing - 1).clamp(min=0).min())
    high = float(((pos - farthest).norm(dim=1) / spacing + 1).max())
    count = max(2 * config.adc_samples, int(16 * (high - low)) + 1)
    response = ofmcw.range_response(config, low, high, count)
    vectors, values, _ = torch.linalg.svd(response, full_matrices=False)
    rank = int((values > torch.finfo(torch.float32).eps / 128 * values[0]).sum())
    return vectors[:, :rank].mH


def refit(config, positions, params, target, adjoint, chunk=32):
    """(coefficients, objective) of the real-coefficient VarPro refit, all in float64."""
    centers, normals = params["centers"].double(), params["normals"].double()
    scale = params["areas"].double().sqrt()
    count = len(centers)
    rank = adjoint.shape[0]
    gram = torch.zeros((count, count), dtype=DTYPE)
    rhs = torch.zeros(count, dtype=DTYPE)
    y_all = target.to(torch.complex128)
    for start in range(0, len(positions), chunk):
        rows = slice(start, min(start + chunk, len(positions)))
        cols = ofmcw.columns(positions[rows], centers, normals, config) * scale  # [a, K, S]
        projected = torch.einsum("rk,aks->ars", adjoint, cols)  # [a, rank, S]
        y = torch.einsum("rk,ak->ar", adjoint, y_all[rows])
        real = torch.view_as_real(projected).permute(0, 1, 3, 2).reshape(-1, count)
        yr = torch.view_as_real(y).reshape(-1)
        gram += real.T @ real
        rhs += real.T @ yr
    size = target.numel()
    gram, rhs = gram / size, rhs / size
    factor, info = torch.linalg.cholesky_ex(gram)
    if int(info) != 0:
        shift = len(gram) * torch.finfo(torch.float32).eps * torch.linalg.eigvalsh(gram)[-1]
        factor = torch.linalg.cholesky(gram + shift * torch.eye(count, dtype=DTYPE))
    b = torch.cholesky_solve(rhs[:, None], factor)[:, 0]
    energy = 0.0
    for start in range(0, len(positions), chunk):
        rows = slice(start, min(start + chunk, len(positions)))
        cols = ofmcw.columns(positions[rows], centers, normals, config) * scale
        prediction = cols @ b.to(torch.complex128)
        energy += float((prediction - y_all[rows]).abs().square().sum())
    del rank
    return b, energy / size


def timed_refit(config, positions, params, target, adjoint, threads=None):
    """Wall seconds of one refit on the given apertures (host cores, float64)."""
    if threads:
        torch.set_num_threads(threads)
    start = time.perf_counter()
    refit(config, positions, params, target, adjoint)
    return time.perf_counter() - start


def timed_solve(count, threads=None):
    """Wall seconds of the float64 Cholesky factor and solve of one [count, count] system."""
    if threads:
        torch.set_num_threads(threads)
    generator = torch.Generator().manual_seed(0)
    m = torch.randn(count, count, generator=generator, dtype=DTYPE)
    h = m @ m.T / count + torch.eye(count, dtype=DTYPE)
    q = torch.randn(count, 1, generator=generator, dtype=DTYPE)
    start = time.perf_counter()
    factor = torch.linalg.cholesky(h)
    torch.cholesky_solve(q, factor)
    return time.perf_counter() - start
