"""Per-stage timing of the DSFW step: NVTX ranges plus CUDA-event durations.

Disabled by default (no cost beyond a flag test). enable() starts recording;
report() returns {stage: [count, milliseconds]} after synchronizing. Stages nest;
each keeps its own total.
"""

from __future__ import annotations

from contextlib import contextmanager

import torch

_records: dict | None = None


def enable():
    global _records
    _records = {}


def disable():
    global _records
    _records = None


@contextmanager
def stage(name):
    if _records is None:
        yield
        return
    torch.cuda.nvtx.range_push(name)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    try:
        yield
    finally:
        end.record()
        torch.cuda.nvtx.range_pop()
        _records.setdefault(name, []).append((start, end))


def report():
    """{stage: [count, total milliseconds]}; synchronizes the device."""
    if not _records:
        return {}
    torch.cuda.synchronize()
    return {name: [len(pairs), round(sum(s.elapsed_time(e) for s, e in pairs), 3)]
            for name, pairs in _records.items()}  # fmt: skip
