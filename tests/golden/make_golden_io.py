"""Generate golden outputs of the reference's experiment I/O helpers.

Run here, where the reference checkout exists (it never exists on the GPU machine):

    python tests/golden/make_golden_io.py /path/to/Dirichlet-Splatting   (or set DSPLAT_REFERENCE)

It imports the reference's examples/evaluation.py (geometry_metrics, write_ply) and
examples/common.py (select_diverse, save_result), runs them on seeded inputs and writes
inputs and outputs to tests/golden/reference_io.npz; tests/test_experiments.py checks
dsplat.experiments against them. Text outputs (the PLY file, the JSON files) are stored
as their bytes.
"""

from __future__ import annotations

import contextlib
import io
import json
import sys
import tempfile
import types
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import torch

HERE = Path(__file__).resolve().parent


def reference_root(args):
    """The reference checkout: the first argument, else $DSPLAT_REFERENCE; there is no default."""
    import os

    value = args[0] if args else os.environ.get("DSPLAT_REFERENCE")
    if not value:
        raise SystemExit("name the reference checkout: an argument or DSPLAT_REFERENCE=/path/to/Dirichlet-Splatting")
    root = Path(value)
    if not (root / "dsplat").is_dir():
        raise SystemExit(f"{root} holds no dsplat package")
    return root


def surface(generator, count, radius, noise):
    """Points on a sphere cap of the given radius, with Gaussian noise (float32)."""
    u = generator.uniform(0.4, 1.0, count)
    phi = generator.uniform(0, 2 * np.pi, count)
    s = np.sqrt(1 - u * u)
    points = radius * np.stack([s * np.cos(phi), s * np.sin(phi), -u], 1) + [0, 0, 0.35]
    return (points + noise * generator.standard_normal(points.shape)).astype(np.float32)


def main(root: Path):
    sys.modules.setdefault("slangtorch", types.ModuleType("slangtorch"))  # the Slang loader is not needed here
    sys.path.insert(0, str(root))
    from dsplat import FMCWConfig, Scan  # noqa: E402
    from examples import common, evaluation  # noqa: E402

    out = {}
    generator = np.random.default_rng(2024)
    # geometry_metrics: recovered clouds of several sizes and noise levels against a truth
    for case, (count, truth_count, noise) in enumerate([(300, 500, 0.0005), (1000, 700, 0.002), (64, 2000, 0.004)]):
        truth = surface(generator, truth_count, 0.03, 0.0)
        points = surface(generator, count, 0.03, noise)
        metrics = evaluation.geometry_metrics(points, truth)
        out[f"metrics{case}_points"] = points
        out[f"metrics{case}_truth"] = truth
        out[f"metrics{case}_keys"] = np.array(list(metrics))
        out[f"metrics{case}_values"] = np.array(list(metrics.values()), dtype=np.float64)
    # select_diverse: quantized scores (ties), 2-D and 3-D candidates, several counts
    for case, (count, dim, wanted, separation) in enumerate([(400, 3, 25, 0.004), (300, 2, 40, 0.05), (50, 3, 0, 0.01)]):
        candidates = generator.uniform(-0.05, 0.05, (count, dim)).astype(np.float32)
        scores = np.round(generator.uniform(0, 1, count), 1).astype(np.float32)
        chosen = common.select_diverse(scores, candidates, wanted, separation)
        out[f"diverse{case}_scores"] = scores
        out[f"diverse{case}_candidates"] = candidates
        out[f"diverse{case}_args"] = np.array([wanted, separation], dtype=np.float64)
        out[f"diverse{case}_chosen"] = np.array(chosen, dtype=np.int64)
    # write_ply with and without normals
    positions = surface(generator, 17, 0.03, 0.001)
    normals = generator.standard_normal((17, 3)).astype(np.float32)
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    with tempfile.TemporaryDirectory() as folder:
        for name, extra in (("ply_plain", None), ("ply_normals", normals)):
            path = Path(folder) / f"{name}.ply"
            evaluation.write_ply(path, positions, extra)
            out[f"{name}_bytes"] = np.frombuffer(path.read_bytes(), dtype=np.uint8)
        out["ply_positions"] = positions
        out["ply_normal_vectors"] = normals
        # save_result on a small state
        params = {"centers": torch.from_numpy(positions), "normals": torch.from_numpy(normals),
                  "areas": torch.full((17,), 2e-5)}  # fmt: skip
        state = SimpleNamespace(params=params, coefficients=torch.linspace(0.1, 1.7, 17),
                                prediction=torch.arange(12, dtype=torch.float32).reshape(3, 4).to(torch.complex64) * (1 + 2j),
                                history=({"iteration": 0, "objective": 1.5, "nmse": 0.25},
                                         {"iteration": 1, "objective": 0.75, "nmse": 0.125, "replaced": 3}))  # fmt: skip
        initial = {"centers": torch.from_numpy(positions[::-1].copy())}
        metrics = {"nmse": 0.125, "surface_median_mm": 1.25, "note": "seeded"}
        with contextlib.redirect_stdout(io.StringIO()) as printed:
            common.save_result(Path(folder), state, initial, metrics)
        with np.load(Path(folder) / "reconstruction.npz") as saved:
            out["save_keys"] = np.array(list(saved.keys()))
        for name in ("reconstruction.ply", "history.json", "metrics.json"):
            out["save_" + name.replace(".", "_")] = np.frombuffer((Path(folder) / name).read_bytes(), dtype=np.uint8)
        out["save_printed"] = np.frombuffer(printed.getvalue().encode(), dtype=np.uint8)
    # progress lines: report every fifth iteration, describe a scan and its chirp
    with contextlib.redirect_stdout(io.StringIO()) as printed:
        for entry in ({"iteration": 10, "nmse": 0.0123456789, "replaced": 2},
                      {"iteration": 11, "nmse": 0.5},
                      {"iteration": 0, "nmse": 1.0, "lm_accepted": 1}):  # fmt: skip
            common.report(entry)
        for config in (FMCWConfig(), FMCWConfig(bandwidth_hz=4e9, adc_samples=128, pad_factor=2)):
            scan = Scan(torch.zeros((64, config.num_range_bins), dtype=torch.complex64),
                        torch.zeros((64, 3)), config)  # fmt: skip
            common.describe(scan)
    out["progress_printed"] = np.frombuffer(printed.getvalue().encode(), dtype=np.uint8)
    np.savez_compressed(HERE / "reference_io.npz", **out)
    print("wrote", HERE / "reference_io.npz", len(out), "arrays", json.dumps(sorted(out)[:4]))


if __name__ == "__main__":
    main(reference_root(sys.argv[1:]))
