"""Many uneven scenes: the persistent multi-scene render and scene-by-scene fitting rounds."""

from __future__ import annotations

import pytest
import torch
from conftest import rel_l2

from oracle import fmcw as ofmcw

pytestmark = pytest.mark.gpu


def _scenes():
    from dsplat.workloads import uneven_scenes

    scenes = uneven_scenes(6, seed=3, device="cuda")
    for scene in scenes:  # keep the float64 oracle quick: trim apertures and surfels
        scene["positions"] = scene["positions"][:300].contiguous()
        for key in ("centers", "normals", "areas", "amplitudes"):
            scene[key] = scene[key][:150].contiguous()
    return scenes


def test_persistent_multi_scene_render_matches_each_scene():
    """One dsg_surfel_render_scenes launch (128 and 256 range bins, ragged tiles, an empty
    surfel set) against the single-scene kernel and the float64 oracle."""
    from dsplat.kernels import surfel as kernel

    scenes = _scenes()
    assert {s["config"].num_range_bins for s in scenes} == {128, 256}
    scenes[2] = dict(scenes[2], centers=scenes[2]["centers"][:0], normals=scenes[2]["normals"][:0],
                     amplitudes=scenes[2]["amplitudes"][:0])  # fmt: skip
    batch = [(s["config"], s["positions"], s["centers"], s["normals"], s["amplitudes"], 0.0) for s in scenes]
    outputs = kernel.render_scenes(batch)
    for scene, out, entry in zip(scenes, outputs, batch, strict=True):
        single = kernel.render(*entry)
        assert out.shape == single.shape == (300, scene["config"].num_range_bins)
        if len(scene["centers"]) == 0:
            assert bool((out == 0).all())
            continue
        assert rel_l2(out, single) < 1e-6
        expected = ofmcw.render(scene["config"], scene["positions"].cpu(), scene["centers"].cpu(),
                                scene["normals"].cpu(), scene["amplitudes"].cpu())  # fmt: skip
        assert rel_l2(out, expected) < 1e-5


def test_multi_scene_render_rejects_an_unsupported_chirp_before_launching():
    from dsplat import FMCWConfig
    from dsplat.kernels import _lib
    from dsplat.kernels import surfel as kernel

    scene = _scenes()[0]
    entry = (FMCWConfig(pad_factor=4), scene["positions"], scene["centers"], scene["normals"], scene["amplitudes"], 0.0)
    before = _lib.library().dsg_launch_count()
    with pytest.raises(_lib.DsplatKernelError):
        kernel.render_scenes([entry])
    assert _lib.library().dsg_launch_count() == before


def test_rounds_of_scenes_follow_each_scene_fitted_alone():
    """Two small scenes stepped in rounds (one step of each, twice) give the histories of
    fitting each scene on its own; the batch NMSE from one launch matches each state's."""
    from dsplat import DSFWConfig, SpatialSearchConfig, initialize, step
    from dsplat.scenes import batch_nmse, fit_scenes, problems_from_scenes
    from dsplat.workloads import uneven_scenes

    scenes = [s for s in uneven_scenes(12, seed=5, device="cuda") if len(s["positions"]) == 1024][:2]
    for scene in scenes:
        for key in ("centers", "normals", "areas", "amplitudes"):
            scene[key] = scene[key][:300].contiguous()
    problems = problems_from_scenes(scenes)
    config = DSFWConfig(iterations=2, batch=64, gram="bf16x3", batched=True)
    search = SpatialSearchConfig(proposal_apertures=256, refine_apertures=512)
    together = fit_scenes(problems, config, search)
    for problem, state in zip(problems, together, strict=True):
        alone = initialize(problem.model, problem.target, problem.start, config, parameters=problem.parameters)
        for _ in range(config.iterations):
            alone = step(alone, config, search)
        for mine, theirs in zip(state.history, alone.history, strict=True):
            assert abs(mine["nmse"] - theirs["nmse"]) <= 1e-6 * max(theirs["nmse"], 1e-12), (mine, theirs)
    for state, nmse in zip(together, batch_nmse(together), strict=True):
        assert abs(nmse - state.history[-1]["nmse"]) <= 1e-4 * state.history[-1]["nmse"] + 1e-9
