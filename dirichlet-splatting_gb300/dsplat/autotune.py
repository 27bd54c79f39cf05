"""Launch-shape autotuner of this library's kernels, with a JSON cache.

The reference fixes its Slang tile constants at import (dsplat/kernels/__init__.py:17-21
PAD, TILE; kernels/surfel.py:42-55). Here the launch shapes that matter on GB300 are knobs
of libdsplat_gb300.so (dsg_tuning_set) or of the bindings, chosen per problem shape by
timing the candidates with CUDA events on the device in use:

  family    knob                              candidates
  splat     DSG_TUNE_SPLAT_CTAS_PER_SM        2, 4, 6, 8, 12 target CTAs per SM of the
                                              segment (render, JVP) and aperture-chunk
                                              (VJP, correlations) splits
  project   DSG_TUNE_PROJECT_STAGES           2, 3, 4 pipeline stages of the fused
                                              design projection (capped by shared memory)
  orient    DSG_TUNE_ORIENT_WARPS             2, 4, 8 warps per CTA of the normal bank
  gram      k splits of dsg_gram_bf16x3       half, once and twice the automatic split

Keys are (family, apertures, surfels, bins, pad, rank2, device name) with apertures and
surfels rounded up to powers of two, so one tuning serves the neighbouring shapes a fit
produces. The cache lives in $DSPLAT_TUNING_CACHE, else dsplat/_build/tuning.json beside
the built library. Without an entry every knob stays automatic (value 0).
"""

from __future__ import annotations

import json
import os
import threading
from pathlib import Path

import torch

KNOBS = {"splat": 0, "project": 1, "orient": 2}  # DSG_TUNE_* of include/dsplat_gb300.h
CANDIDATES = {"splat": (2, 4, 6, 8, 12), "project": (2, 3, 4), "orient": (2, 4, 8)}

_lock = threading.Lock()
_cache: dict | None = None
_applied: dict = {}


def cache_path() -> Path:
    override = os.environ.get("DSPLAT_TUNING_CACHE")
    if override:
        return Path(override)
    return Path(__file__).resolve().parent / "_build" / "tuning.json"


def _bucket(n):
    """n rounded up to a power of two (0 stays 0)."""
    n = int(n)
    return 0 if n <= 0 else 1 << (n - 1).bit_length()


_DEVICE_NAMES: dict = {}


def _device_name(device):
    if device is None or not torch.cuda.is_available():
        return "any"
    index = torch.device(device).index
    index = torch.cuda.current_device() if index is None else index
    name = _DEVICE_NAMES.get(index)
    if name is None:
        name = _DEVICE_NAMES[index] = torch.cuda.get_device_name(index)
    return name


def shape_key(family, apertures=0, surfels=0, bins=0, pad=0, rank2=0, device=None):
    """The cache key of a problem shape."""
    name = _device_name(device)
    return f"{family}|A{_bucket(apertures)}|S{_bucket(surfels)}|K{int(bins)}|P{int(pad)}|R{int(rank2)}|{name}"


def _load():
    global _cache
    if _cache is None:
        path = cache_path()
        try:
            _cache = json.loads(path.read_text()) if path.exists() else {}
        except (OSError, json.JSONDecodeError):
            _cache = {}
    return _cache


def _save():
    path = cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    temporary = path.with_suffix(".tmp")
    temporary.write_text(json.dumps(_load(), indent=1, sort_keys=True))
    temporary.replace(path)


def reset(memory_only=False):
    """Forget the loaded cache (and the applied knobs); the next lookup reads the file again."""
    global _cache
    with _lock:
        _cache = None
        _applied.clear()
        if not memory_only:
            path = cache_path()
            if path.exists():
                path.unlink()


def lookup(key):
    """The tuned value of a key, or None."""
    with _lock:
        entry = _load().get(key)
    return None if entry is None else int(entry["value"])


def record(key, value, timings):
    """Store a tuned value with the timings it was chosen from."""
    with _lock:
        _load()[key] = {"value": int(value), "ms": {str(k): round(float(v), 5) for k, v in timings.items()}}
        _save()


def set_knob(family, value):
    """Set a library knob (0: automatic) unless it already holds that value."""
    if _applied.get(family) == value:
        return
    from .kernels import _lib

    _lib.call("dsg_tuning_set", KNOBS[family], int(value))
    _applied[family] = value


def apply(family, **shape):
    """Set the knob of a family from the cache for this shape (automatic when untuned)."""
    value = lookup(shape_key(family, **shape))
    set_knob(family, value or 0)


def choose(candidates, measure):
    """(best candidate, {candidate: ms}) by measure(candidate) -> milliseconds (smallest wins)."""
    timings = {candidate: float(measure(candidate)) for candidate in candidates}
    best = min(timings, key=lambda c: (timings[c], c))
    return best, timings


def time_cuda(function, repeats=3, warmup=1):
    """Median milliseconds of function() over repeats, CUDA events on the current stream."""
    for _ in range(warmup):
        function()
    samples = []
    for _ in range(repeats):
        begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        begin.record()
        function()
        end.record()
        end.synchronize()
        samples.append(begin.elapsed_time(end))
    return sorted(samples)[len(samples) // 2]


def tune_knob(family, key, run, candidates=None, repeats=3):
    """Time run() under every candidate value of a library knob, keep and record the best."""
    candidates = candidates or CANDIDATES[family]

    def measure(value):
        set_knob(family, value)
        return time_cuda(run, repeats=repeats)

    best, timings = choose(candidates, measure)
    set_knob(family, best)
    record(key, best, timings)
    return best, timings


def gram_splits(automatic, key):
    """The tuned k-split count of a Gram launch, or the automatic one."""
    value = lookup(key)
    return automatic if value is None else value


@torch.no_grad()
def tune_workload(config, positions, params, residual, basis=None, fresnel_n=0.0):
    """Tune every family on the shapes of a DSFW fit of these apertures and surfels.

    Returns {family: (chosen value, {candidate: ms})}. Every measured launch computes a
    full result with that candidate's launch shape; the results do not depend on it
    beyond the order of the float sums.
    """
    from .certificate import fibonacci_sphere
    from .fmcw import FMCWModel, Scan
    from .kernels import surfel as kernel

    device = positions.device
    A, S, K = len(positions), len(params["centers"]), config.num_range_bins
    centers, normals = params["centers"], params["normals"]
    weights = params["areas"].sqrt().to(torch.complex64)
    upstream = residual.reshape(A, K)
    chosen = {}

    def splat():
        kernel.render(config, positions, centers, normals, weights, fresnel_n)
        kernel.vjp(config, positions, centers, normals, weights, upstream, fresnel_n)

    chosen["splat"] = tune_knob("splat", shape_key("splat", A, S, K, config.pad_factor, device=device), splat)
    sub = positions[: min(A, 384)].contiguous()
    grid = centers.repeat(-(-50000 // S), 1)[:50000].contiguous()
    grid_n = normals.repeat(-(-50000 // S), 1)[:50000].contiguous()
    bank = fibonacci_sphere(24, device)
    table = FMCWModel(Scan(upstream[: len(sub)], sub, config)).range_table(upstream[: len(sub)], 8)

    def orient():
        kernel.correlate_orientations(config, sub, grid, grid_n, bank, upstream[: len(sub)], fresnel_n, table)

    orient_key = shape_key("orient", len(sub), 0, K, config.pad_factor, device=device)
    chosen["orient"] = tune_knob("orient", orient_key, orient)
    if basis is not None:
        from .kernels.gram import GramRows, append_projected, fused_supported

        if fused_supported(config, basis):
            first = positions[: min(A, 2048)].contiguous()
            rank2 = basis.interleaved.shape[0]
            store = GramRows(S, len(first) * rank2, device)
            status = torch.zeros(1, dtype=torch.int32, device=device)

            def project():
                store.rows = 0
                append_projected(store, config, first, params, basis, fresnel_n, status)

            project_key = shape_key("project", 0, S, K, config.pad_factor, rank2, device)
            chosen["project"] = tune_knob("project", project_key, project)
            chosen["gram"] = _tune_gram(S, device)
    return chosen


def _tune_gram(columns, device, rows=200_000):
    """k splits of the normal-equation Gram (columns unknowns) on rows random projected rows."""
    from .kernels.gram import GramRows, check, k_splits

    generator = torch.Generator(device=device).manual_seed(0)
    store = GramRows(columns, rows, device)
    store.append(torch.randn(rows, columns, device=device, generator=generator))
    total = torch.zeros((columns, columns), dtype=torch.float64, device=device)
    automatic = k_splits(store.n_pad, store.k_pad)
    key = gram_key(store.n_pad, store.k_pad, 0, device)
    candidates = sorted({max(1, automatic // 2), automatic, automatic * 2})

    def measure(splits):
        return time_cuda(lambda: check(store.accumulate(total, splits=splits)))

    best, timings = choose(candidates, measure)
    record(key, best, timings)
    return best, timings


def gram_key(n_pad, k_pad, column_from, device):
    """Cache key of a Gram launch: unknowns, row bucket, and whether it is a cross product."""
    return shape_key("gram", apertures=k_pad, surfels=n_pad, rank2=int(column_from > 0), device=device)
