"""End-to-end DSFW fits on the GPU with the bars of the reference's own experiment tests.

The reference checks its experiments at small presets (tests/test_examples.py:28-41):
every fit's objective never rises, the 2-D spectrum fit recovers every tone (NMSE < 1e-6,
center RMSE < 0.01 bins), and the planar raster fit from a migration start reaches
NMSE < 1e-4. The same properties are asserted here on scenes built by this package
(the star outline of dsplat.workloads, a planar set of point reflectors), plus the C2
workload at full size (256^2 grid, 80 tones at 20 dB SNR) for a few steps and several
uneven FMCW scenes (the C5 configuration, scaled down) one after another in batched mode.
"""

from __future__ import annotations

import itertools
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


def _monotone(history):
    return all(b["objective"] <= a["objective"] * (1 + 1e-6) for a, b in itertools.pairwise(history))


def _assignment_rmse(found, truth, period):
    from scipy.optimize import linear_sum_assignment

    delta = found.double().cpu()[:, None] - truth.double().cpu()[None]
    delta = delta - period * torch.round(delta / period)
    cost = delta.square().sum(-1)
    rows, cols = linear_sum_assignment(cost.numpy())
    return float(cost[rows, cols].mean().sqrt())


@pytest.mark.parametrize("window", ["rect", "hann"])
def test_spectral_fit_recovers_every_tone(window):
    """24 x 24 grid, 4 noiseless tones on the star outline, 14 steps (the smoke preset)."""
    from dsplat import DSFWConfig, ParameterConfig, SpectralGrid, SpectralModel, fit

    side, count = 24, 4
    grid = SpectralGrid((side, side), window=window)
    generator = torch.Generator().manual_seed(0)
    truth = (side / 2 + 0.4 * side * _star(count)).cuda()
    amplitudes = torch.polar(torch.ones(count, dtype=torch.float64),
                             2 * math.pi * torch.rand(count, generator=generator, dtype=torch.float64))  # fmt: skip
    target = _windowed_spectrum(side, truth.double().cpu(), amplitudes, window).cuda()
    start = {"centers": (torch.rand(count, 2, generator=generator) * side).cuda()}
    config = DSFWConfig(iterations=14, ridge=1e-8, coefficients="complex", replacement="utility",
                        min_separation=0.35, lm_solver="dense", lm_steps=3, lm_rows=grid.size,
                        lm_gain_ratio=0, screen_apertures=0, trust_radius=0.75)  # fmt: skip
    state = fit(SpectralModel(grid), target, start, config, candidates={"centers": grid.bins()},
                parameters={"centers": ParameterConfig(period=grid.shape)})  # fmt: skip
    assert _monotone(state.history)
    assert state.history[-1]["nmse"] < 1e-6
    assert _assignment_rmse(state.params["centers"], truth, side) < 1e-2


def test_c2_star_spectrum_fit_improves_monotonically():
    """C2 at full size: 256^2, 80 tones on the star at 20 dB SNR, 80 random atoms, 20
    steps. Utility replacement exchanges one atom per step, so 20 steps explain about a
    quarter of the 80 tones: the NMSE must fall below 0.9 (measured 0.925 after 6 steps)."""
    from dsplat import DSFWConfig, ParameterConfig, SpectralGrid, SpectralModel, initialize, step
    from dsplat.workloads import star_tones

    grid = SpectralGrid((256, 256))
    target, truth = star_tones()
    generator = torch.Generator().manual_seed(1)
    start = {"centers": (torch.rand(80, 2, generator=generator) * 256).cuda()}
    config = DSFWConfig(iterations=20, ridge=1e-8, coefficients="complex", replacement="utility",
                        min_separation=0.35, lm_solver="dense", lm_steps=3, lm_rows=grid.size,
                        lm_gain_ratio=0, screen_apertures=0, trust_radius=0.75)  # fmt: skip
    state = initialize(SpectralModel(grid), target, start, config, candidates={"centers": grid.bins()},
                       parameters={"centers": ParameterConfig(period=grid.shape)})  # fmt: skip
    for _ in range(20):
        state = step(state, config)
    history = state.history
    assert _monotone(history)
    assert history[-1]["nmse"] < 0.9 and history[-1]["nmse"] < history[0]["nmse"]
    assert all(entry.get("replaced", 1) <= 1 for entry in history)  # utility: one slot per step


def test_planar_fit_from_a_migration_start():
    """The planar raster experiment at its smoke size: a 24 x 24 raster at a quarter
    wavelength (4 GHz chirp), a plane of candidate points 16 x 16 over +-40 mm at 0.35 m,
    ten reflectors on candidate points; migration scores the candidates, the 24 strongest
    start a fit of in-plane centers with utility replacement over the candidate points, and
    after 12 steps the NMSE is below 1e-4 with an objective that never rose."""
    from dsplat import DSFWConfig, FMCWConfig, FMCWModel, ParameterConfig, fit
    from dsplat.fmcw import migration
    from dsplat.groundtruth import planar_array, synthesize

    sensor = FMCWConfig(bandwidth_hz=4e9, adc_samples=128, pad_factor=2, sweep_time_s=20e-6)
    positions = planar_array(24, sensor.lambda_m / 4, device="cuda")
    axis = torch.linspace(-0.04, 0.04, 16, device="cuda")
    x, y = torch.meshgrid(axis, axis, indexing="ij")
    points = torch.stack([x.flatten(), y.flatten(), torch.full_like(x.flatten(), 0.35)], -1)
    lit = [3 * 16 + 3, 3 * 16 + 12, 5 * 16 + 7, 6 * 16 + 8, 7 * 16 + 9, 8 * 16 + 5, 9 * 16 + 10, 10 * 16 + 4,
           12 * 16 + 12, 13 * 16 + 2]  # fmt: skip
    truth = points[lit]
    normals = torch.tensor([0.0, 0.0, -1.0], device="cuda").expand(len(lit), 3).contiguous()
    weights = torch.full((len(lit),), 1 / len(lit) ** 0.5, device="cuda", dtype=torch.complex64)
    scan = synthesize(positions, truth, normals, weights, sensor)
    scores = migration(scan, points, (24, 24), padding=8).abs()
    start_ids = scores.argsort(descending=True)[:24]
    area = (0.08 / 15) ** 2
    params = {"centers": points[start_ids].clone(), "normals": normals[:1].expand(24, 3).clone(),
              "areas": torch.full((24,), area, device="cuda")}  # fmt: skip
    parameters = {"centers": ParameterConfig(trainable=(True, True, False), scale=0.001, lower=(-0.04, -0.04, 0.35),
                                             upper=(0.04, 0.04, 0.35)),
                  "normals": ParameterConfig(trainable=False, normalize=True),
                  "areas": ParameterConfig(trainable=False)}  # fmt: skip
    config = DSFWConfig(iterations=12, ridge=1e-14 * area, coefficients="complex", replacement="utility",
                        min_separation=0.0005, lm_solver="dense", lm_steps=2, lm_rows=128 * scan.data.shape[1],
                        lm_gain_ratio=0, screen_apertures=0)  # fmt: skip
    state = fit(FMCWModel(scan), scan.data, params, config, candidates={"centers": points}, parameters=parameters)
    assert _monotone(state.history)
    assert state.history[-1]["nmse"] < 1e-4


def test_uneven_fmcw_scenes_fit_one_after_another_in_batched_mode():
    """C5 scaled down: four scenes with different array sides, ADC lengths and surfel
    counts on ellipsoid caps, three batched mixed-precision steps each; every objective
    falls monotonically and none of the scenes disturbs the next (graph caches keyed by
    shape)."""
    from dsplat import DSFWConfig, FMCWConfig, FMCWModel, ParameterConfig, SpatialSearchConfig, initialize, step
    from dsplat.groundtruth import planar_array, synthesize
    from dsplat.workloads import box_of, random_start

    scenes = [(32, 128, 200, 0.30), (48, 256, 350, 0.40), (32, 256, 150, 0.45), (64, 128, 500, 0.35)]
    for index, (side, samples, count, depth) in enumerate(scenes):
        config = FMCWConfig(adc_samples=samples)
        positions = planar_array(side, 0.0025, standoff=depth, device="cuda")
        generator = torch.Generator().manual_seed(10 + index)
        axes = 0.015 + 0.025 * torch.rand(3, generator=generator, dtype=torch.float64)
        u = 1 - 0.6 * torch.rand(count, generator=generator, dtype=torch.float64)  # cap: -n_z in [0.4, 1]
        phi = 2 * math.pi * torch.rand(count, generator=generator, dtype=torch.float64)
        s = (1 - u.square()).sqrt()
        sphere = torch.stack([s * phi.cos(), s * phi.sin(), -u], -1)
        centers = (torch.tensor([0.0, 0.0, depth], dtype=torch.float64) + axes * sphere).float().cuda()
        normals = torch.nn.functional.normalize(sphere / axes, dim=1).float().cuda()
        areas = torch.full((count,), 2 * math.pi * float(axes.mean()) ** 2 * 0.6 / count, device="cuda")
        amplitudes = areas.sqrt().to(torch.complex64)
        scan = synthesize(positions, centers, normals, amplitudes, config)
        low, high = box_of(centers, 0.005)
        start = random_start(count, low, high, float(areas[0]), seed=index, device="cuda")
        parameters = {"centers": ParameterConfig(scale=5e-4, lower=low, upper=high),
                      "normals": ParameterConfig(scale=0.1, normalize=True), "areas": ParameterConfig(trainable=False)}  # fmt: skip
        dsfw = DSFWConfig(iterations=3, batch=128, gram="bf16x3", batched=True)
        search = SpatialSearchConfig(proposal_apertures=256, refine_apertures=512)
        state = initialize(FMCWModel(scan), scan.data, start, dsfw, parameters=parameters)
        for _ in range(3):
            state = step(state, dsfw, search)
        assert _monotone(state.history), (index, state.history)
        assert state.history[-1]["nmse"] < state.history[0]["nmse"], (index, state.history)


def _star(count):
    from dsplat.workloads import _STAR, _outline

    return torch.tensor(_outline(_STAR, count), dtype=torch.float32)


def _windowed_spectrum(side, centers, amplitudes, window):
    """Spectrum [side, side] of complex tones sampled in float64 under a separable taper."""
    t = torch.arange(side, dtype=torch.float64)
    samples = torch.zeros((side, side), dtype=torch.complex128)
    for c, b in zip(centers, amplitudes, strict=True):
        samples += b * torch.exp(2j * math.pi * (c[0] * t[:, None] + c[1] * t[None, :]) / side)
    if window == "rect":
        taper = torch.ones(side, dtype=torch.float64)
    else:
        taper = torch.hann_window(side, periodic=True, dtype=torch.float64)
    samples = samples * taper[:, None] * taper[None] / taper.sum().square()
    return torch.fft.fftn(samples).to(torch.complex64)
