"""Experiment I/O (dsplat.experiments) against the reference's own outputs.

tests/golden/reference_io.npz holds what the reference's examples/evaluation.py and
examples/common.py produced on seeded inputs (tests/golden/make_golden_io.py): surface
metrics, diverse selections, PLY files, a saved result folder and the progress lines.
Host-side only.
"""

from __future__ import annotations

import contextlib
import io
import json
from dataclasses import dataclass
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest
import torch

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_io.npz")


def _text(key):
    return bytes(GOLDEN[key]).decode()


@pytest.mark.parametrize("case", [0, 1, 2])
def test_geometry_metrics_match_the_reference(case):
    from dsplat.experiments import geometry_metrics

    metrics = geometry_metrics(GOLDEN[f"metrics{case}_points"], GOLDEN[f"metrics{case}_truth"])
    assert list(metrics) == list(GOLDEN[f"metrics{case}_keys"])
    np.testing.assert_allclose(list(metrics.values()), GOLDEN[f"metrics{case}_values"], rtol=1e-12, atol=0)


def test_geometry_metrics_by_brute_force():
    """Nearest distances by an all-pairs search give the same figures as the tree queries."""
    from dsplat.experiments import geometry_metrics

    generator = np.random.default_rng(7)
    points = generator.uniform(0, 0.01, (40, 3))
    truth = generator.uniform(0, 0.01, (55, 3))
    distances = np.linalg.norm(points[:, None] - truth[None], axis=2)
    forward, backward = distances.min(1), distances.min(0)
    precision, recall = np.mean(forward < 0.002), np.mean(backward < 0.002)
    metrics = geometry_metrics(points, truth)
    assert metrics["surface_median_mm"] == pytest.approx(np.median(forward) * 1000, rel=1e-12)
    assert metrics["chamfer_mm"] == pytest.approx((forward.mean() + backward.mean()) * 500, rel=1e-12)
    assert metrics["fscore_2mm"] == pytest.approx(2 * precision * recall / (precision + recall), rel=1e-12)


@pytest.mark.parametrize("case", [0, 1, 2])
def test_select_diverse_matches_the_reference(case):
    """Ties (scores rounded to tenths) go highest index first; count 0 still keeps one."""
    from dsplat.experiments import select_diverse

    wanted, separation = GOLDEN[f"diverse{case}_args"]
    chosen = select_diverse(GOLDEN[f"diverse{case}_scores"], GOLDEN[f"diverse{case}_candidates"], int(wanted),
                            float(separation))  # fmt: skip
    assert chosen == GOLDEN[f"diverse{case}_chosen"].tolist()


@pytest.mark.parametrize("name,with_normals", [("ply_plain", False), ("ply_normals", True)])
def test_ply_bytes_match_and_read_back(tmp_path, name, with_normals):
    from dsplat.experiments import read_ply, write_ply

    positions, normals = GOLDEN["ply_positions"], GOLDEN["ply_normal_vectors"]
    path = tmp_path / "cloud.ply"
    write_ply(path, positions, normals if with_normals else None)
    assert path.read_bytes() == bytes(GOLDEN[f"{name}_bytes"])
    read_positions, read_normals = read_ply(path)
    assert np.array_equal(read_positions.astype(np.float32), positions)  # 9 digits round-trip float32
    if with_normals:
        assert np.array_equal(read_normals.astype(np.float32), normals)
    else:
        assert read_normals is None


def test_empty_and_foreign_ply(tmp_path):
    from dsplat.experiments import read_ply, write_ply

    write_ply(tmp_path / "empty.ply", np.zeros((0, 3)))
    positions, normals = read_ply(tmp_path / "empty.ply")
    assert positions.shape == (0, 3) and normals is None
    (tmp_path / "binary.ply").write_text("ply\nformat binary_little_endian 1.0\nend_header\n")
    with pytest.raises(ValueError):
        read_ply(tmp_path / "binary.ply")


def test_save_result_writes_the_reference_folder(tmp_path):
    from dsplat.experiments import save_result

    positions, normals = GOLDEN["ply_positions"], GOLDEN["ply_normal_vectors"]
    params = {"centers": torch.from_numpy(positions), "normals": torch.from_numpy(normals),
              "areas": torch.full((17,), 2e-5)}  # fmt: skip
    state = SimpleNamespace(params=params, coefficients=torch.linspace(0.1, 1.7, 17),
                            prediction=torch.arange(12, dtype=torch.float32).reshape(3, 4).to(torch.complex64) * (1 + 2j),
                            history=({"iteration": 0, "objective": 1.5, "nmse": 0.25},
                                     {"iteration": 1, "objective": 0.75, "nmse": 0.125, "replaced": 3}))  # fmt: skip
    initial = {"centers": torch.from_numpy(positions[::-1].copy())}
    metrics = {"nmse": 0.125, "surface_median_mm": 1.25, "note": "seeded"}
    with contextlib.redirect_stdout(io.StringIO()) as printed:
        save_result(tmp_path, state, initial, metrics)
    assert printed.getvalue() == _text("save_printed")
    with np.load(tmp_path / "reconstruction.npz") as saved:
        assert list(saved.keys()) == list(GOLDEN["save_keys"])
        assert np.array_equal(saved["initial_centers"], positions[::-1])
        assert np.array_equal(saved["prediction"], state.prediction.numpy())
    for name in ("reconstruction.ply", "history.json", "metrics.json"):
        assert (tmp_path / name).read_bytes() == bytes(GOLDEN["save_" + name.replace(".", "_")]), name


def test_a_planar_result_has_no_point_cloud(tmp_path):
    """Spectral fits have 2-D centers: no PLY, the rest as usual."""
    from dsplat.experiments import save_result

    state = SimpleNamespace(params={"centers": torch.rand(5, 2)}, coefficients=torch.ones(5),
                            prediction=torch.zeros(4, 4), history=())  # fmt: skip
    with contextlib.redirect_stdout(io.StringIO()):
        save_result(tmp_path, state, {}, {})
    assert not (tmp_path / "reconstruction.ply").exists()
    assert json.loads((tmp_path / "history.json").read_text()) == []


@dataclass(frozen=True)
class _Preset:
    side: int = 24
    window: str = "hann"


def test_output_folder_records_arguments_and_configs(tmp_path):
    from dsplat.experiments import output, parser

    args = parser("signal2d", {"demo": None, "smoke": None}).parse_args(
        ["--preset", "smoke", "--seed", "3", "--output", str(tmp_path / "run")])  # fmt: skip
    folder = output(args, preset=_Preset(), extra=np.float32(1.5))
    recorded = json.loads((folder / "configuration.json").read_text())
    assert recorded["arguments"]["preset"] == "smoke" and recorded["arguments"]["seed"] == 3
    assert recorded["preset"] == {"side": 24, "window": "hann"}
    assert recorded["extra"] == "1.5"
    default = parser("raw2d", {"demo": None}).parse_args([])
    assert default.preset == "demo" and default.iterations is None and default.output is None


def test_progress_lines_match_the_reference():
    """report every fifth iteration and describe of two chirps, as the reference prints them."""
    from dsplat import FMCWConfig, Scan
    from dsplat.experiments import describe, report

    with contextlib.redirect_stdout(io.StringIO()) as printed:
        for entry in ({"iteration": 10, "nmse": 0.0123456789, "replaced": 2},
                      {"iteration": 11, "nmse": 0.5},
                      {"iteration": 0, "nmse": 1.0, "lm_accepted": 1}):  # fmt: skip
            report(entry)
        for config in (FMCWConfig(), FMCWConfig(bandwidth_hz=4e9, adc_samples=128, pad_factor=2)):
            describe(Scan(torch.zeros((64, config.num_range_bins), dtype=torch.complex64), torch.zeros((64, 3)),
                          config))  # fmt: skip
    assert printed.getvalue() == _text("progress_printed")
