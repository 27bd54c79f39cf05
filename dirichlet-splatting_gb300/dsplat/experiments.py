"""Experiment outputs of the render-and-fit path: result folders, point clouds and metrics.

The reference's experiments write one folder per run (examples/common.py:13-43: the
argument parser, ``output`` with configuration.json, ``save_result`` with
reconstruction.npz, reconstruction.ply, history.json and metrics.json), print progress
(:46-63 ``report``, ``describe``), pick diverse starting points (:66-77
``select_diverse``) and score recovered surfaces against the truth
(examples/evaluation.py:7-30 ``geometry_metrics``, ``write_ply``). The file names, npz
keys, JSON layout and the ASCII PLY header are the reference's, so tools that read its
outputs read these. Everything here is host-side NumPy/SciPy; ``read_ply`` is added for
round trips. The reference's matplotlib figures are not produced (matplotlib is not a
dependency of this package).
"""

from __future__ import annotations

import argparse
import json
from dataclasses import asdict, is_dataclass
from pathlib import Path

import numpy as np

__all__ = [
    "parser", "output", "save_result", "report", "describe", "select_diverse",
    "geometry_metrics", "write_ply", "read_ply", "write_json",
]  # fmt: skip


def parser(experiment, presets):
    """Command line of an experiment: preset, seed, iteration and ridge overrides, output folder."""
    result = argparse.ArgumentParser(description=f"{experiment}: an experiment on the dsplat library")
    result.set_defaults(experiment=experiment)
    result.add_argument("--preset", choices=list(presets), default="demo")
    result.add_argument("--seed", type=int, default=0)
    result.add_argument("--iterations", type=int)
    result.add_argument("--ridge", type=float)
    result.add_argument("--output")
    return result


def write_json(path, value):
    """Indented JSON; dataclasses (configs) as dictionaries, anything else unknown as text."""

    def fallback(item):
        return asdict(item) if is_dataclass(item) else str(item)

    Path(path).write_text(json.dumps(value, indent=2, default=fallback), encoding="utf-8")


def output(args, **config):
    """The run's folder (``--output``, else outputs/<experiment>_<preset>_seed<seed>), created,
    with the arguments and configuration recorded in configuration.json."""
    folder = Path(args.output or f"outputs/{args.experiment}_{args.preset}_seed{args.seed}")
    folder.mkdir(parents=True, exist_ok=True)
    write_json(folder / "configuration.json", {"arguments": vars(args), **config})
    return folder


def save_result(path, state, initial, metrics):
    """reconstruction.npz (final and initial parameters, coefficients, prediction), a PLY of
    the centers when they are 3-D, history.json and metrics.json; prints the metrics."""
    path = Path(path)
    arrays = {key: _host(value) for key, value in state.params.items()}
    for key, value in initial.items():
        arrays["initial_" + key] = _host(value)
    arrays["coefficients"] = _host(state.coefficients)
    arrays["prediction"] = _host(state.prediction)
    np.savez_compressed(path / "reconstruction.npz", **arrays)
    if arrays["centers"].shape[1] == 3:
        write_ply(path / "reconstruction.ply", arrays["centers"], arrays.get("normals"))
    write_json(path / "history.json", state.history)
    write_json(path / "metrics.json", metrics)
    print(json.dumps(metrics, indent=2), flush=True)


def report(entry):
    """One progress line every fifth DSFW iteration."""
    if entry["iteration"] % 5:
        return
    print(f"DSFW {entry['iteration']:4d} NMSE {entry['nmse']:.6g} replaced={entry.get('replaced', 0)} "
          f"LM={entry.get('lm_accepted', 0)}", flush=True)  # fmt: skip


def describe(scan):
    """Print the scan's dimensions and its chirp."""
    chirp = scan.fmcw_config
    apertures, bins = scan.data.shape
    kind = str(scan.data.dtype).removeprefix("torch.")
    print(f"scan       {kind} [{apertures}, {bins}]: {apertures} apertures x {bins} positive range bins")
    print(f"chirp      {chirp.fc_hz / 1e9:g} GHz carrier, {chirp.bandwidth_hz / 1e9:g} GHz bandwidth, "
          f"{chirp.adc_samples} ADC samples, FFT length {chirp.n_fft}, "
          f"{chirp.range_bin_spacing_m * 1000:.2f} mm per range bin", flush=True)  # fmt: skip


def select_diverse(scores, candidates, count, min_separation):
    """Greedy best-first indices at least min_separation apart (NumPy arrays).

    Candidates are visited in reversed stable ascending order of score, so equal scores go
    highest index first; a candidate closer than min_separation to a kept one is skipped.
    The count is checked after each kept candidate, so the best candidate is kept even for
    count <= 0, as in the reference.
    """
    candidates = np.asarray(candidates)
    chosen = []
    kept = np.empty((0,) + candidates.shape[1:], dtype=candidates.dtype)
    for index in np.argsort(np.asarray(scores), kind="stable")[::-1]:
        point = candidates[index]
        if len(kept) and np.linalg.norm(kept - point, axis=1).min() < min_separation:
            continue
        chosen.append(int(index))
        kept = np.concatenate([kept, point[None]])
        if len(chosen) >= count:
            break
    return chosen


def geometry_metrics(points, reference, threshold_m=0.002):
    """Accuracy (recovered to truth) and completeness (truth to recovered) of a surface.

    Nearest-neighbour distances both ways give the median and mean surface distance of the
    recovered points (mm), the Chamfer distance (mean of both directions, mm), and the
    fractions within threshold_m: precision, recall and their F-score.
    """
    from scipy.spatial import cKDTree

    to_truth = cKDTree(reference).query(points)[0]
    to_recovered = cKDTree(points).query(reference)[0]
    precision = float(np.mean(to_truth < threshold_m))
    recall = float(np.mean(to_recovered < threshold_m))
    return {
        "surface_median_mm": float(np.median(to_truth) * 1000),
        "surface_mean_mm": float(to_truth.mean() * 1000),
        "chamfer_mm": float((to_truth.mean() + to_recovered.mean()) * 500),
        "precision_2mm": precision,
        "recall_2mm": recall,
        "fscore_2mm": 2 * precision * recall / max(precision + recall, 1e-30),
    }


_PLY_AXES = ("x", "y", "z")
_PLY_NORMALS = ("nx", "ny", "nz")


def write_ply(path, positions, normals=None):
    """ASCII PLY of float vertices (positions in metres, optional unit normals), 9 digits."""
    names = _PLY_AXES + (_PLY_NORMALS if normals is not None else ())
    header = ["ply", "format ascii 1.0", f"element vertex {len(positions)}"]
    header += [f"property float {name}" for name in names]
    header.append("end_header")
    rows = np.asarray(positions) if normals is None else np.hstack([positions, normals])
    with open(path, "w", encoding="ascii") as file:
        file.write("\n".join(header) + "\n")
        np.savetxt(file, rows, fmt="%.9g")


def read_ply(path):
    """positions [N, 3] and normals [N, 3] (or None) of an ASCII PLY written by write_ply."""
    with open(path, encoding="ascii") as file:
        if file.readline().strip() != "ply" or file.readline().strip() != "format ascii 1.0":
            raise ValueError(f"{path}: not an ASCII PLY file")
        count, names = 0, []
        for line in file:
            words = line.split()
            if words[:2] == ["element", "vertex"]:
                count = int(words[2])
            elif words[:1] == ["property"]:
                names.append(words[-1])
            elif words[:1] == ["end_header"]:
                break
        values = np.loadtxt(file, ndmin=2, max_rows=count) if count else np.empty((0, len(names)))
    columns = {name: values[:, i] for i, name in enumerate(names)}
    positions = np.stack([columns[name] for name in _PLY_AXES], axis=1)
    normals = np.stack([columns[name] for name in _PLY_NORMALS], axis=1) if "nx" in columns else None
    return positions, normals


def _host(value):
    return value.detach().cpu().numpy() if hasattr(value, "detach") else np.asarray(value)
