"""Shared fixtures. GPU tests carry the `gpu` marker; everything else runs on the CPU.

The package under test is dirichlet-splatting_gb300/dsplat (a drop-in for the
reference's `dsplat`); oracle/ is the float64 CPU checker.
"""

from __future__ import annotations

import sys
from pathlib import Path

import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent
for path in (ROOT, ROOT / "dirichlet-splatting_gb300"):
    if str(path) not in sys.path:
        sys.path.insert(0, str(path))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the sm_103a library")


def pytest_collection_modifyitems(config, items):
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def close(actual, expected, tolerance=2e-5):
    """Agreement within tolerance times the largest expected magnitude."""
    expected = expected.to(actual.device, actual.dtype)
    atol = tolerance * float(expected.abs().max())
    torch.testing.assert_close(actual, expected, rtol=0, atol=atol)


def rel_l2(actual, expected):
    """Relative L2 error of actual against expected, computed in float64 on the CPU."""
    a = actual.detach().cpu().to(torch.complex128 if actual.is_complex() else torch.float64)
    e = expected.detach().cpu().to(a.dtype)
    return float((a - e).norm() / e.norm().clamp(min=1e-300))


def aperture_grid(side=8, pitch=0.004, device="cuda"):
    t = (torch.arange(side, dtype=torch.float32) - (side - 1) / 2) * pitch
    x, y = torch.meshgrid(t, t, indexing="ij")
    return torch.stack([x.flatten(), y.flatten(), torch.zeros(side * side)], -1).to(device)


def surfels(count, seed=0, spread=0.01, device="cuda"):
    """Surfels near (0, 0, 0.3) facing the apertures at z = 0."""
    generator = torch.Generator().manual_seed(seed)
    centers = torch.tensor([0, 0, 0.3]) + spread * (2 * torch.rand(count, 3, generator=generator) - 1)
    direction = torch.tensor([0.0, 0, -1]) + 0.3 * torch.randn(count, 3, generator=generator)
    normals = torch.nn.functional.normalize(direction, dim=1)
    areas = torch.full((count,), 1e-4)
    return {k: v.to(device) for k, v in dict(centers=centers, normals=normals, areas=areas).items()}


def fmcw_specs(trainable_normals=True):
    from dsplat import ParameterConfig

    return dict(
        centers=ParameterConfig(scale=0.0005, lower=(-0.02, -0.02, 0.28), upper=(0.02, 0.02, 0.32)),
        normals=ParameterConfig(trainable=trainable_normals, scale=0.1, normalize=True),
        areas=ParameterConfig(trainable=False),
    )


@pytest.fixture
def fmcw():
    """An 8x8-aperture scan of five surfels with real reflectivities, rendered on the GPU."""
    from dsplat import FMCWConfig, FMCWModel, Scan

    config = FMCWConfig()
    positions = aperture_grid()
    params = surfels(5)
    coefficients = torch.linspace(0.5, 1.5, 5, device="cuda")
    empty = Scan(torch.zeros((len(positions), config.num_range_bins), dtype=torch.complex64,
                             device="cuda"), positions, config)  # fmt: skip
    data = FMCWModel(empty).render(params, coefficients)
    return FMCWModel(Scan(data, positions, config)), params, coefficients


@pytest.fixture
def spectral():
    """Three complex tones on a 24 x 20 periodic grid, one exactly on a bin."""
    from dsplat import SpectralGrid, SpectralModel

    grid = SpectralGrid((24, 20))
    centers = torch.tensor([[3.3, 4.1], [12.0, 15.0], [18.4, 7.9]], device="cuda")
    coefficients = torch.tensor([1 + 0.5j, -0.7 + 0.2j, 0.4 - 0.9j], device="cuda")
    return SpectralModel(grid), {"centers": centers}, coefficients
