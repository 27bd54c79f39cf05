"""Seeded synthetic workloads of the benchmark configurations.

The reference publishes no benchmark data; these generators stand in for its scenes
with the stated shapes, sizes and value distributions:

forward_scene   32 x 32 array at 2.5 mm pitch (z = 0, facing +z), 256 surfels with
                centers uniform in [-20, 20]^2 x [330, 370] mm and normals uniform on
                the hemisphere facing -z, amplitude sqrt(1e-6 m^2).
sphere_cap      128 x 128 array at 2.5 mm pitch, 2000 surfels area-uniform on the
                front hemisphere of a 30 mm sphere centred at (0, 0, 0.35) m, outward
                normals, amplitude sqrt(cap area / 2000).
random_start    the fit's initial surfels: centers uniform in the box plus a 5 mm
                margin, Gaussian-normalized normals, frozen areas.
star_tones      80 unit tones along a five-point star spanning 60 % of a 256^2 grid,
                uniform phases, complex Gaussian noise at 20 dB SNR.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .groundtruth import planar_array


def forward_scene(surfel_count=256, side=32, seed=0, device="cuda"):
    """(positions [A, 3], params, weights [S] complex) of the small forward workload."""
    generator = torch.Generator().manual_seed(seed)
    lo = torch.tensor([-0.02, -0.02, 0.33])
    hi = torch.tensor([0.02, 0.02, 0.37])
    centers = lo + (hi - lo) * torch.rand(surfel_count, 3, generator=generator)
    normals = torch.nn.functional.normalize(torch.randn(surfel_count, 3, generator=generator), dim=1)
    normals[:, 2] = -normals[:, 2].abs()
    areas = torch.full((surfel_count,), 1e-6)
    params = {k: v.to(device) for k, v in dict(centers=centers, normals=normals, areas=areas).items()}
    positions = planar_array(side, 0.0025, device=device)
    weights = torch.ones(surfel_count, dtype=torch.complex64, device=device) * math.sqrt(1e-6)
    return positions, params, weights


def sphere_cap(surfel_count=2000, side=128, radius=0.03, depth=0.35, seed=0, device="cuda"):
    """(positions, params, reflectivities [S]) of the 128^2-array, 2000-surfel sphere cap."""
    generator = torch.Generator().manual_seed(seed)
    t = torch.rand(surfel_count, generator=generator, dtype=torch.float64)  # -n_z, uniform: equal area
    phi = 2 * math.pi * torch.rand(surfel_count, generator=generator, dtype=torch.float64)
    ring = (1 - t.square()).clamp(min=0).sqrt()
    normals = torch.stack((ring * phi.cos(), ring * phi.sin(), -t), -1)
    centers = torch.tensor([0.0, 0.0, depth], dtype=torch.float64) + radius * normals
    area = 2 * math.pi * radius * radius / surfel_count
    params = {
        "centers": centers.float().to(device),
        "normals": normals.float().to(device),
        "areas": torch.full((surfel_count,), area, device=device),
    }
    positions = planar_array(side, 0.0025, device=device)
    reflectivity = torch.ones(surfel_count, device=device)
    return positions, params, reflectivity


def box_of(centers, margin=0.005):
    """Lower and upper corners (lists) of the centers' bounding box plus a margin."""
    low = (centers.min(0).values - margin).tolist()
    high = (centers.max(0).values + margin).tolist()
    return low, high


def random_start(count, low, high, area, seed=0, device="cuda"):
    """Initial surfels: centers uniform in [low, high], Gaussian-normalized normals."""
    generator = torch.Generator().manual_seed(seed)
    lo, hi = torch.tensor(low), torch.tensor(high)
    centers = lo + (hi - lo) * torch.rand(count, 3, generator=generator)
    normals = torch.nn.functional.normalize(torch.randn(count, 3, generator=generator), dim=1)
    return {
        "centers": centers.to(device),
        "normals": normals.to(device),
        "areas": torch.full((count,), float(area), device=device),
    }


_STAR = [
    (math.sin(2 * math.pi * k / 10) * (1 if k % 2 == 0 else 0.38),
     math.cos(2 * math.pi * k / 10) * (1 if k % 2 == 0 else 0.38))
    for k in range(11)
]  # fmt: skip


def _outline(points, count):
    """count points evenly spaced by arc length along a closed polyline, from its first vertex."""
    vertices = np.asarray(points, dtype=np.float64)
    lengths = np.linalg.norm(np.diff(vertices, axis=0), axis=1)
    ends = np.cumsum(lengths)
    out = []
    for s in np.arange(count) * ends[-1] / count:
        i = int(np.searchsorted(ends, s))
        start = ends[i] - lengths[i]
        out.append(vertices[i] + (vertices[i + 1] - vertices[i]) * (s - start) / lengths[i])
    return np.stack(out)


def star_tones(side=256, count=80, span=0.3, snr_db=20.0, seed=0, device="cuda"):
    """(target [side, side] complex64, true centers [count, 2] in bins) of the star spectrum.

    Tones at side / 2 + span * side * outline, synthesized in float64 as sampled
    complex exponentials and FFT'd; noise at the given SNR.
    """
    generator = torch.Generator().manual_seed(seed)
    xy = torch.tensor(_outline(_STAR, count), dtype=torch.float64)
    truth = side / 2 + span * side * xy
    phases = 2 * math.pi * torch.rand(count, generator=generator, dtype=torch.float64)
    amplitudes = torch.polar(torch.ones(count, dtype=torch.float64), phases)
    t = torch.arange(side, dtype=torch.float64)
    samples = torch.zeros((side, side), dtype=torch.complex128)
    for c, b in zip(truth, amplitudes, strict=True):
        samples += b * torch.exp(2j * math.pi * (c[0] * t[:, None] + c[1] * t[None, :]) / side)
    target = torch.fft.fftn(samples / (side * side))
    power = target.abs().square().mean()
    sigma = (power / 10 ** (snr_db / 10) / 2).sqrt()
    noise = torch.complex(torch.randn(side, side, generator=generator, dtype=torch.float64),
                          torch.randn(side, side, generator=generator, dtype=torch.float64))  # fmt: skip
    target = target + sigma * noise
    return target.to(torch.complex64).to(device), truth.float().to(device)


def uneven_scenes(count=64, seed=0, device="cuda"):
    """count FMCW scenes of uneven size (the batched many-scene workload), seeded.

    Each scene draws: array side from {32, 64, 96, 128} at 2.5 mm pitch; 128 or 256 ADC
    samples (pad 2, so 128 or 256 range bins); 200 to 4000 surfels area-uniform on the front
    (n_z < 0) half of an ellipsoid with semi-axes 15-40 mm centred at depth 0.30-0.45 m, with
    outward normals and reflectivity one. Returns a list of dicts with the FMCWConfig, the
    positions, the true surfels (centers, normals, areas) and their amplitudes.
    """
    from .fmcw import FMCWConfig

    generator = torch.Generator().manual_seed(seed)
    scenes = []
    for _ in range(count):
        side = (32, 64, 96, 128)[int(torch.randint(0, 4, (1,), generator=generator))]
        samples = (128, 256)[int(torch.randint(0, 2, (1,), generator=generator))]
        surfels = int(torch.randint(200, 4001, (1,), generator=generator))
        axes = 0.015 + 0.025 * torch.rand(3, generator=generator, dtype=torch.float64)
        depth = 0.30 + 0.15 * float(torch.rand(1, generator=generator, dtype=torch.float64))
        # area-uniform on the unit sphere's front half, then stretched onto the ellipsoid
        z = torch.rand(surfels, generator=generator, dtype=torch.float64)
        phi = 2 * math.pi * torch.rand(surfels, generator=generator, dtype=torch.float64)
        ring = (1 - z.square()).clamp(min=0).sqrt()
        unit = torch.stack((ring * phi.cos(), ring * phi.sin(), -z), -1)
        centers = torch.tensor([0.0, 0.0, depth], dtype=torch.float64) + axes * unit
        normals = torch.nn.functional.normalize(unit / axes, dim=1)  # ellipsoid normal ~ gradient of x^2/a^2
        mean_axis = float(axes.mean())
        area = 2 * math.pi * mean_axis * mean_axis / surfels
        scenes.append({
            "config": FMCWConfig(adc_samples=samples),
            "positions": planar_array(side, 0.0025, device=device),
            "centers": centers.float().to(device),
            "normals": normals.float().to(device),
            "areas": torch.full((surfels,), area, device=device),
            "amplitudes": torch.full((surfels,), math.sqrt(area), dtype=torch.complex64, device=device),
        })  # fmt: skip
    return scenes
