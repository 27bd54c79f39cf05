"""The seeded synthetic workloads that stand in for the reference's scenes, on the CPU.

bench.py and the fit tests build their inputs with dsplat.workloads; these checks pin the
shapes, sizes and distributions the module states (array pitch, sphere-cap geometry and
area, start box, star outline, noise level) and that the same seed gives the same data.
"""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch


def test_sphere_cap_lies_on_the_front_hemisphere_with_outward_normals():
    from dsplat.workloads import sphere_cap

    positions, params, reflectivity = sphere_cap(surfel_count=500, side=16, device="cpu")
    centers, normals = params["centers"].double(), params["normals"].double()
    center = torch.tensor([0.0, 0.0, 0.35], dtype=torch.float64)
    assert torch.allclose((centers - center).norm(dim=1), torch.full((500,), 0.03, dtype=torch.float64), atol=1e-7)
    assert torch.allclose(normals.norm(dim=1), torch.ones(500, dtype=torch.float64), atol=1e-6)
    assert torch.allclose((centers - center) / 0.03, normals, atol=1e-5)  # outward
    assert bool((normals[:, 2] <= 0).all())  # facing the array at z = 0
    # -n_z uniform on [0, 1] (equal area): mean 1/2, variance 1/12
    assert abs(float(-normals[:, 2].mean()) - 0.5) < 0.05
    assert abs(float(normals[:, 2].var()) - 1 / 12) < 0.015
    assert float(params["areas"].sum()) == pytest.approx(2 * math.pi * 0.03**2, rel=1e-5)
    assert positions.shape == (256, 3) and torch.equal(reflectivity, torch.ones(500))


def test_planar_array_pitch_and_centre():
    from dsplat.groundtruth import planar_array

    positions = planar_array(4, 0.0025).double()
    assert positions.shape == (16, 3)
    assert torch.allclose(positions.mean(0), torch.zeros(3, dtype=torch.float64), atol=1e-12)
    x = torch.unique(positions[:, 0].round(decimals=9))
    assert torch.allclose(torch.diff(x), torch.full((3,), 0.0025, dtype=torch.float64), atol=1e-9)
    assert float(positions[:, 2].abs().max()) == 0.0


def test_random_start_fills_the_box_plus_margin():
    from dsplat.workloads import box_of, random_start

    centers = torch.tensor([[0.0, -0.01, 0.33], [0.01, 0.02, 0.36]])
    low, high = box_of(centers, 0.005)
    assert low == pytest.approx([-0.005, -0.015, 0.325]) and high == pytest.approx([0.015, 0.025, 0.365])
    start = random_start(4000, low, high, 1e-6, seed=3, device="cpu")
    c = start["centers"]
    assert bool((c >= torch.tensor(low)).all()) and bool((c <= torch.tensor(high)).all())
    assert torch.allclose(c.mean(0), (torch.tensor(low) + torch.tensor(high)) / 2, atol=1e-3)
    assert torch.allclose(start["normals"].norm(dim=1), torch.ones(4000), atol=1e-6)
    assert torch.equal(start["areas"], torch.full((4000,), 1e-6))
    again = random_start(4000, low, high, 1e-6, seed=3, device="cpu")
    assert all(torch.equal(start[k], again[k]) for k in start)


def test_star_outline_is_evenly_spaced_and_the_noise_at_the_stated_snr():
    from dsplat.workloads import _STAR, _outline, star_tones

    points = _outline(_STAR, 80)
    closed = np.vstack([points, points[:1]])
    steps = np.linalg.norm(np.diff(closed, axis=0), axis=1)
    perimeter = np.linalg.norm(np.diff(np.asarray(_STAR), axis=0), axis=1).sum()
    # chords across a vertex are shorter than the arc-length step; none is longer
    assert steps.max() == pytest.approx(perimeter / 80, rel=1e-9)
    assert np.median(steps) == pytest.approx(perimeter / 80, rel=1e-6)
    target, truth = star_tones(side=64, count=20, snr_db=20.0, device="cpu")
    assert target.shape == (64, 64) and target.dtype == torch.complex64 and truth.shape == (20, 2)
    assert float(truth.min()) >= 64 * (0.5 - 0.3) - 1e-4 and float(truth.max()) <= 64 * (0.5 + 0.3) + 1e-4
    clean, _ = star_tones(side=64, count=20, snr_db=200.0, device="cpu")
    noise = (target - clean).abs().square().mean()
    assert float(clean.abs().square().mean() / noise) == pytest.approx(100.0, rel=0.15)


def test_forward_scene_ranges():
    from dsplat.workloads import forward_scene

    positions, params, weights = forward_scene(device="cpu")
    c = params["centers"]
    assert positions.shape == (1024, 3) and c.shape == (256, 3)
    assert float(c[:, :2].abs().max()) <= 0.02 and 0.33 <= float(c[:, 2].min()) and float(c[:, 2].max()) <= 0.37
    assert bool((params["normals"][:, 2] <= 0).all())
    assert torch.allclose(weights.abs(), torch.full((256,), 1e-3))
