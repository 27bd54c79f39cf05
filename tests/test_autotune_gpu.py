"""The autotuner on the GPU: every candidate launch shape gives the same results, the chosen
knobs reach the library, and the JSON cache is written and read back."""

from __future__ import annotations

import pytest
import torch
from conftest import rel_l2

from oracle import fmcw as ofmcw

pytestmark = pytest.mark.gpu


@pytest.fixture
def tuning_cache(tmp_path, monkeypatch):
    from dsplat import autotune

    monkeypatch.setenv("DSPLAT_TUNING_CACHE", str(tmp_path / "tuning.json"))
    autotune.reset(memory_only=True)
    yield tmp_path / "tuning.json"
    for family in autotune.KNOBS:
        autotune.set_knob(family, 0)
    autotune.reset(memory_only=True)


def test_every_splat_launch_shape_matches_the_oracle(tuning_cache):
    """Render and VJP under each candidate segment / chunk split: same values as the float64 oracle."""
    from dsplat import FMCWConfig, autotune
    from dsplat.kernels import _lib
    from dsplat.kernels import surfel as kernel
    from dsplat.workloads import forward_scene

    positions, params, weights = forward_scene()
    config = FMCWConfig()
    expected = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), weights.cpu())
    for value in autotune.CANDIDATES["splat"]:
        autotune.set_knob("splat", value)
        assert _lib.query("dsg_tuning_get", autotune.KNOBS["splat"]) == value
        out = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
        assert rel_l2(out, expected) < 1e-5, value


def test_tuned_workload_records_every_family_and_applies_it(tuning_cache):
    from dsplat import FMCWConfig, FMCWModel, ParameterConfig, Scan, autotune
    from dsplat.kernels import _lib
    from dsplat.workloads import box_of, sphere_cap

    config = FMCWConfig()
    positions, params, _ = sphere_cap(side=32, surfel_count=300, device="cuda")
    generator = torch.Generator().manual_seed(0)
    residual = torch.complex(torch.randn(len(positions), 128, generator=generator),
                             torch.randn(len(positions), 128, generator=generator)).cuda()  # fmt: skip
    low, high = box_of(params["centers"])
    model = FMCWModel(Scan(residual, positions, config)).prepare({"centers": ParameterConfig(lower=low, upper=high)})
    basis = model.block_basis(slice(0, len(positions) * 128))
    chosen = autotune.tune_workload(config, positions, params, residual, basis)
    assert set(chosen) >= {"splat", "orient"}
    for family, (value, timings) in chosen.items():
        assert value in timings and all(t > 0 for t in timings.values()), (family, timings)
    assert tuning_cache.exists()
    autotune.reset(memory_only=True)  # read back from the file
    autotune.set_knob("splat", 0)
    autotune.apply("splat", apertures=len(positions), surfels=300, bins=128, pad=2, device=positions.device)
    assert _lib.query("dsg_tuning_get", autotune.KNOBS["splat"]) == chosen["splat"][0]
