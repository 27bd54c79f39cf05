"""Whole DSFW fits on the GPU against the reference solver's own histories.

tests/golden/reference_fits.json holds the objective / NMSE history, the replacement
counts and the final centers of the reference's unmodified Python solver (dsplat/dsfw.py
and the modules under it), run on the CPU with its kernel bindings computed by the float64
oracle (tests/golden/make_golden_fits.py). The same scene code runs here through the GB300
package on CUDA, so the records differ only by the implementation: float32 kernels in a
different summation order against float64 ones.

The reference itself is re-run with every model-kernel output perturbed by relative noise
of 1e-6 and 1e-5 (the rounding of float32 kernels); "spread" records how far those runs
move. Bars, step by step: the replacement count is one the reference runs produced; the
NMSE lies within the reference runs' range widened by 5 % (or below 1e-9, float32
round-off of an exact fit). Every final reference center has one of ours within 50 um or
within twice the reference runs' own center scatter, whichever is larger.
"""

from __future__ import annotations

import importlib.util
import json
from pathlib import Path

import pytest
import torch

GOLDEN = Path(__file__).resolve().parent / "golden"
REFERENCE = json.loads((GOLDEN / "reference_fits.json").read_text())
NMSE_RELATIVE = 0.05
NMSE_FLOOR = 1e-9
CENTER_TOL_M = 5e-5


def _scenes():
    spec = importlib.util.spec_from_file_location("make_golden_fits", GOLDEN / "make_golden_fits.py")
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module.run_scenes


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("name", sorted(REFERENCE))
def test_fit_follows_the_reference_solver(name, batched):
    """Plain mode, and batched mode (DSFWConfig(batched=True): device elimination from the
    inverse factor, fused certificate ascent, refined shifted solves), against the same
    reference records and bands."""
    from dataclasses import replace

    import dsplat

    configure = (lambda cfg: replace(cfg, batched=True)) if batched else None
    ours = _scenes()(dsplat, "cuda", names={name}, configure=configure)[name]
    theirs = REFERENCE[name]
    assert len(ours["history"]) == len(theirs["history"])
    spread = theirs["spread"]
    for mine, ref, band in zip(ours["history"], theirs["history"], spread["steps"], strict=True):
        assert mine.get("replaced", -1.0) in band["replaced"], (name, mine, ref, band)
        low = band["nmse_min"] * (1 - NMSE_RELATIVE) - NMSE_FLOOR
        high = band["nmse_max"] * (1 + NMSE_RELATIVE) + NMSE_FLOOR
        assert low <= mine["nmse"] <= high, (name, mine, ref, band)
    mine_c = torch.tensor(ours["centers"], dtype=torch.float64)
    ref_c = torch.tensor(theirs["centers"], dtype=torch.float64)
    assert mine_c.shape == ref_c.shape
    nearest = torch.cdist(ref_c, mine_c).min(dim=1).values
    assert float(nearest.max()) < max(CENTER_TOL_M, 2 * spread["center_scatter_m"]), (name, nearest.tolist())


def test_reference_records_are_complete():
    """The committed records cover every scene and each starts from iteration 0."""
    assert set(REFERENCE) == {"fmcw_merged_joint", "fmcw_merged_dense", "fmcw_nearby_joint",
                              "fmcw_spatial_search", "spectral_utility_dense"}  # fmt: skip
    for record in REFERENCE.values():
        assert record["history"][0]["iteration"] == 0
        assert all("nmse" in e and "objective" in e for e in record["history"])
        assert len(record["spread"]["steps"]) == len(record["history"])
