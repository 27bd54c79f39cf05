"""The headline fit's accuracy: mixed+batched against the plain FP32 drop-in, 100 steps.

The 128^2-array, 2000-surfel sphere-cap fit (batch 256, SpatialSearchConfig()) from two
seeded scenes and starts, run in both arithmetics: the plain FP32 arm (FP32 SSYRK Gram,
the reference's structure) and the mixed+batched arm (split-BF16x3 tcgen05 Gram with the
coefficients refined against the rendered residual, device-resident search and
replacement loops).

A fit is a chaotic sequence of discrete decisions: the final NMSE of one run moves by
10-25 % when nothing but the launch shapes (the order of float sums) change, in either
arm; the median centre-to-surface distance moves by a few per cent. So the arms are
compared on their means over the seeds: the mixed arm's mean median distance within 5 %
of the plain arm's, and its mean final NMSE within the run-to-run spread (15 %). Over
three seeds the mixed arm's mean NMSE was 14 % lower and its distance 4 % higher
(bench.py --accuracy 3). This file is collected late: it takes about three minutes.
"""

from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

DISTANCE_TOLERANCE = 0.05
NMSE_TOLERANCE = 0.15
SEEDS = (0, 1)


def test_mixed_arm_is_as_accurate_as_plain_after_100_steps():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch

    import bench
    from dsplat import DSFWConfig, SpatialSearchConfig, initialize, step

    device = torch.device("cuda", 0)
    search = SpatialSearchConfig()
    arms = {"plain": DSFWConfig(iterations=100, batch=256),
            "mixed": DSFWConfig(iterations=100, batch=256, gram="bf16x3", batched=True)}  # fmt: skip
    finals = {name: [] for name in arms}
    for seed in SEEDS:
        model, target, start, parameters, truth = bench.build_problem(device, seed=seed)
        for name, config in arms.items():
            state = initialize(model, target, start, config, parameters=parameters)
            for _ in range(config.iterations):
                state = step(state, config, search)
            finals[name].append(bench._fit_figures(state, truth))

    def mean(name, key):
        return sum(entry[key] for entry in finals[name]) / len(finals[name])

    assert mean("mixed", "median_center_to_surface_m") <= mean("plain", "median_center_to_surface_m") * (
        1 + DISTANCE_TOLERANCE), finals  # fmt: skip
    assert mean("mixed", "nmse") <= mean("plain", "nmse") * (1 + NMSE_TOLERANCE), finals
