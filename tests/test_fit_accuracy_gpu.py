"""The headline fit's accuracy: mixed+batched against the plain FP32 drop-in, 100 steps.

The 128^2-array, 2000-surfel sphere-cap fit (batch 256, SpatialSearchConfig()) from one
seeded random start, run in both arithmetics: the plain FP32 arm (FP32 SSYRK Gram, the
reference's structure) and the mixed+batched arm (split-BF16x3 tcgen05 Gram with the
coefficients refined against the rendered residual, device-resident search and
replacement loops). The bar: after 100 steps the mixed arm's data NMSE and its median
centre-to-surface distance are each no more than 5 % above the plain arm's. A fit is a
chaotic sequence of discrete decisions, so the two arms end in different states; over
three seeds the mixed arm's final NMSE was 14 % lower on average and its distance within
4 % (bench.py --accuracy 3).
"""

from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

TOLERANCE = 0.05


def test_mixed_arm_is_no_less_accurate_than_plain_after_100_steps():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch

    import bench
    from dsplat import DSFWConfig, SpatialSearchConfig, initialize, step

    device = torch.device("cuda", 0)
    model, target, start, parameters, truth = bench.build_problem(device)
    search = SpatialSearchConfig()
    finals = {}
    for name, config in {"plain": DSFWConfig(iterations=100, batch=256),
                         "mixed": DSFWConfig(iterations=100, batch=256, gram="bf16x3", batched=True)}.items():
        state = initialize(model, target, start, config, parameters=parameters)
        for _ in range(config.iterations):
            state = step(state, config, search)
        finals[name] = bench._fit_figures(state, truth)
    for key in ("nmse", "median_center_to_surface_m"):
        assert finals["mixed"][key] <= finals["plain"][key] * (1 + TOLERANCE), (key, finals)
