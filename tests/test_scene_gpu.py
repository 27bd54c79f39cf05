"""The composed range/Doppler/azimuth renderer (dsplat.surfel.render_scene) on the GPU.

Values and the gradients of all thirteen surfel quantities are compared with the
reference's own float64 renderer (tests/reference/physics.py), whose outputs
tests/golden/reference_scene.npz holds.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch
from conftest import rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_scene.npz")
KEYS = ("positions", "normals", "areas", "reflectivity", "velocities", "impedance")
CASES = (("rect", (32, 16, 8), "rect"), ("hann", (24, 12, 6), "hann"))


@pytest.mark.parametrize("name,shape,window", CASES)
def test_scene_and_its_gradients_match_the_reference_renderer(name, shape, window):
    """float64 inputs: the cube within 1e-5 and every gradient within 1e-4 (rel-L2); the
    atoms are evaluated by the float32 spectral kernel and its hand-written VJP."""
    from dsplat.surfel import Sensor, render_scene

    inputs = [torch.from_numpy(GOLDEN[f"{name}_{k}"]).cuda().requires_grad_() for k in KEYS]
    gamma = float(GOLDEN[f"{name}_meta"][0])
    cube = render_scene(*inputs, Sensor(shape=shape), gamma=gamma, window=window)
    expected = torch.from_numpy(GOLDEN[f"{name}_cube"])
    assert cube.shape == shape
    assert rel_l2(cube, expected) < 1e-5
    upstream = torch.from_numpy(GOLDEN[f"{name}_upstream"]).cuda()
    grads = torch.autograd.grad((upstream.conj() * cube).real.sum(), inputs)
    for key, grad in zip(KEYS, grads, strict=True):
        assert rel_l2(grad, torch.from_numpy(GOLDEN[f"{name}_grad_{key}"])) < 1e-4, key


def test_float32_scene_is_limited_by_the_carrier_phase_only():
    """float32 inputs against the float64 oracle on the same (rounded) inputs: at 1.5 m the
    round-trip phase 4 pi r / lambda is about 4800 rad, so float32 carries it to ~3e-4 rad."""
    from dsplat.spectral import SpectralGrid
    from dsplat.surfel import Sensor, render_scene

    from oracle import scene

    inputs = [torch.from_numpy(GOLDEN[f"rect_{k}"]) for k in KEYS]
    single = [x.to(torch.complex64 if x.is_complex() else torch.float32) for x in inputs]
    sensor = Sensor(shape=(32, 16, 8))
    cube = render_scene(*[x.cuda() for x in single], sensor)
    expected = scene.render_scene(*single, sensor, SpectralGrid(sensor.shape))
    assert rel_l2(cube, expected) < 2e-3


def test_surfels_facing_away_or_matched_contribute_nothing():
    from dsplat.surfel import Sensor, render_scene

    inputs = [torch.from_numpy(GOLDEN[f"rect_{k}"]).cuda() for k in KEYS]
    positions, normals, areas, reflectivity, velocities, impedance = inputs
    sensor = Sensor(shape=(32, 16, 8))
    # normals along +position face away from the sensor at the origin: cos <= 0
    away = render_scene(positions, positions, areas, reflectivity, velocities, impedance, sensor)
    assert float(away.abs().max()) == 0.0
    lit = render_scene(positions, normals, areas, reflectivity, velocities, impedance, sensor)
    matched = render_scene(positions, normals, areas, reflectivity, velocities, torch.ones_like(impedance), sensor)
    assert float(matched.abs().max()) < 1e-6 * float(lit.abs().max())
