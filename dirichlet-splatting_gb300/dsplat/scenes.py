"""Many uneven FMCW scenes fitted side by side.

A production batch holds scenes of different array sizes, chirps and surfel counts. Their
DSFW fits are independent, so they advance in rounds: every round steps each scene once
(one DSFW step with that scene's shapes; the per-shape CUDA graphs of the certificate
ascent are kept across rounds), and the scenes' profiles are rendered together, all
scenes in one persistent launch (dsg_surfel_render_scenes: a device work queue over
(scene, aperture tile)), whenever every scene's prediction is wanted at once — at the
start, to score the batch, and at the end. No counterpart in the reference, which fits
one scene per call (dsplat/dsfw.py:153-174).
"""

from __future__ import annotations

from dataclasses import dataclass

import torch

from .dsfw import initialize, step
from .fmcw import FMCWModel
from .groundtruth import synthesize
from .kernels import surfel as kernel
from .parameters import ParameterConfig
from .workloads import box_of, random_start


@dataclass
class SceneProblem:
    """One scene of a batch: its model (scan), data, start and constraints."""

    model: FMCWModel
    target: torch.Tensor
    start: dict
    parameters: dict


def problems_from_scenes(scenes, seed=0):
    """SceneProblems of uneven_scenes(): the float64-synthesized scans and seeded starts."""
    problems = []
    for index, scene in enumerate(scenes):
        scan = synthesize(scene["positions"], scene["centers"], scene["normals"], scene["amplitudes"],
                          scene["config"])  # fmt: skip
        low, high = box_of(scene["centers"], 0.005)
        start = random_start(len(scene["centers"]), low, high, float(scene["areas"][0]), seed=seed + index,
                             device=scene["centers"].device)  # fmt: skip
        parameters = {"centers": ParameterConfig(scale=5e-4, lower=low, upper=high),
                      "normals": ParameterConfig(scale=0.1, normalize=True),
                      "areas": ParameterConfig(trainable=False)}  # fmt: skip
        problems.append(SceneProblem(FMCWModel(scan), scan.data, start, parameters))
    return problems


def render_states(states):
    """Every state's prediction, all scenes in one launch (dsg_surfel_render_scenes)."""
    batch = []
    for state in states:
        config, positions = state.model.sensor
        params = state.params
        weights = state.coefficients.to(torch.complex64) * params["areas"].sqrt()
        batch.append((config, positions, params["centers"], params["normals"], weights, state.model.fresnel_n))
    return kernel.render_scenes(batch)


def batch_nmse(states):
    """Data NMSE of every scene's current fit from one batched render (float64 sums)."""
    predictions = render_states(states)
    out = []
    for state, prediction in zip(states, predictions, strict=True):
        residual = (prediction - state.target).to(torch.complex128)
        out.append(residual.abs().square().sum() / state.target.to(torch.complex128).abs().square().sum())
    return [float(value) for value in torch.stack(out).tolist()]


def fit_scenes(problems, config, search=None, rounds=None, callback=None):
    """Initialize every scene, then rounds of one DSFW step per scene; the final states.

    callback(round, states) runs after every round.
    """
    states = [initialize(p.model, p.target, p.start, config, parameters=p.parameters) for p in problems]
    for index in range(config.iterations if rounds is None else rounds):
        states = [step(state, config, search) for state in states]
        if callback is not None:
            callback(index, states)
    return states
