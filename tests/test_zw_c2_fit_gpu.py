"""The full-size 2-D spectrum fit (C2) against the reference solver's own 100-step run.

Workload: 256 x 256 band-limited Fourier samples, 80 unit tones on a five-point star at 20 dB
SNR (dsplat.workloads.star_tones, seed 0), 80 atoms started at random (seed 1), 100 steps
of utility replacement over every grid bin with three dense LM steps each.
tests/golden/make_golden_c2.py ran the reference's unmodified DSFW solver on the same inputs
on the CPU (its kernel bindings replaced by the float64 oracle), once exactly and once with
every model-kernel output perturbed by 1e-6 relative noise (the reference's own spread).

Bars: the final NMSE within 5 % of the reference's (or of its perturbed run, whichever is
nearer), every step's NMSE inside the band of the two reference runs widened by 5 %, and the
fitted tones' centres as close to the truth as the reference's (assignment RMSE in bins,
within 5 % or 0.01 bins). This file is collected late: it takes about half a minute.
"""

from __future__ import annotations

import json
from pathlib import Path

import pytest
import torch

pytestmark = pytest.mark.gpu

RECORD = Path(__file__).parent / "golden" / "reference_c2_fit.json"
TOLERANCE = 0.05


def _assignment_rmse(found, truth, period):
    from scipy.optimize import linear_sum_assignment

    delta = torch.as_tensor(found, dtype=torch.float64).cpu()[:, None] - torch.as_tensor(truth, dtype=torch.float64)[None]
    delta = delta - period * torch.round(delta / period)
    cost = delta.square().sum(-1)
    rows, cols = linear_sum_assignment(cost.numpy())
    return float(cost[rows, cols].mean().sqrt())


@pytest.mark.parametrize("batched", [False, True])
def test_c2_fit_follows_the_reference_solver(batched):
    from dsplat import DSFWConfig, ParameterConfig, SpectralGrid, SpectralModel, initialize, step
    from dsplat.workloads import star_tones

    if not RECORD.exists():
        pytest.skip("tests/golden/reference_c2_fit.json not generated (tests/golden/make_golden_c2.py)")
    records = json.loads(RECORD.read_text())
    exact, noisy = records["exact"], records["noise"]
    grid = SpectralGrid((256, 256))
    target, truth = star_tones(device="cpu")
    generator = torch.Generator().manual_seed(1)
    start = {"centers": (torch.rand(80, 2, generator=generator) * 256).cuda()}
    config = DSFWConfig(iterations=100, ridge=1e-8, coefficients="complex", replacement="utility",
                        min_separation=0.35, lm_solver="dense", lm_steps=3, lm_rows=grid.size,
                        lm_gain_ratio=0, screen_apertures=0, trust_radius=0.75, batched=batched)  # fmt: skip
    state = initialize(SpectralModel(grid), target.cuda(), start, config, candidates={"centers": grid.bins()},
                       parameters={"centers": ParameterConfig(period=grid.shape)})  # fmt: skip
    for _ in range(100):
        state = step(state, config)
    mine = [entry["nmse"] for entry in state.history]
    band = [(min(a["nmse"], b["nmse"]), max(a["nmse"], b["nmse"])) for a, b in zip(exact["history"], noisy["history"],
                                                                                   strict=True)]  # fmt: skip
    assert len(mine) == len(band) == 101
    final = mine[-1]
    nearest = min(abs(final - exact["history"][-1]["nmse"]) / exact["history"][-1]["nmse"],
                  abs(final - noisy["history"][-1]["nmse"]) / noisy["history"][-1]["nmse"])  # fmt: skip
    assert nearest <= TOLERANCE, (final, exact["history"][-1]["nmse"], noisy["history"][-1]["nmse"])
    for i, (value, (low, high)) in enumerate(zip(mine, band, strict=True)):
        assert low * (1 - TOLERANCE) <= value <= high * (1 + TOLERANCE), (i, value, low, high)
    reference_rmse = _assignment_rmse(exact["centers"], truth, 256)
    rmse = _assignment_rmse(state.params["centers"], truth, 256)
    assert rmse <= max(reference_rmse * (1 + TOLERANCE), reference_rmse + 0.01), (rmse, reference_rmse)
