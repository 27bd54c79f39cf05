"""CUDA-graph capture inside the solver's steps.

torch.cuda.graph synchronizes the device and empties PyTorch's caching allocator (device
and pinned host) before every capture, so that the graph's private pool can take as much
memory as possible. Inside a DSFW step that flush costs more than the capture: the large
blocks it frees (Gram row stores, pooled systems) are requested again a few launches
later, and each request then becomes a cudaMalloc that synchronizes the device. recording
captures the same way (a side stream ordered after the current one, a private memory
pool per graph) without the flush.
"""

from __future__ import annotations

from collections import OrderedDict
from contextlib import contextmanager

import torch


_SIDE_STREAMS: dict = {}


def side_stream(device=None, lane=0):
    """One of this device's fixed second streams for work beside the current stream.

    A fixed stream per (device, lane), not a new one per use: PyTorch's caching allocator
    keeps the blocks freed by a stream for that stream, so work that allocates gigabytes
    (Gram row stores) on ever new streams would take new device memory every time. Lane 0
    carries the large speculative work (full normal equations, screening refits); lane 1 the
    short speculative factorizations, so that they never queue behind lane 0.
    """
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    stream = _SIDE_STREAMS.get((device.index, lane))
    if stream is None:
        stream = torch.cuda.Stream(device)
        _SIDE_STREAMS[(device.index, lane)] = stream
    return stream


@contextmanager
def recording(graph):
    """Capture the launches of the block into graph (a torch.cuda.CUDAGraph)."""
    current = torch.cuda.current_stream()
    side = side_stream(current.device)
    side.wait_stream(current)
    with torch.cuda.stream(side):
        graph.capture_begin()
        try:
            yield graph
        finally:
            graph.capture_end()
    current.wait_stream(side)


class GraphCache:
    """Captured graphs (with their static buffers) by shape key, the most recently used kept.

    Every captured graph holds a private memory pool; a process that fits many differently
    shaped problems would otherwise keep one pool per shape forever. The bound is above the
    shapes one batch of scenes cycles through (the many-scene workload steps 64 scenes of
    different surfel counts in rounds, each with its own conjugate-gradient graph), so a
    round replays every scene's graphs instead of capturing them again.
    """

    def __init__(self, limit=128):
        self.limit = limit
        self.entries = OrderedDict()

    def get(self, key):
        entry = self.entries.get(key)
        if entry is not None:
            self.entries.move_to_end(key)
        return entry

    def __setitem__(self, key, entry):
        self.entries[key] = entry
        self.entries.move_to_end(key)
        while len(self.entries) > self.limit:
            self.entries.popitem(last=False)

    def __len__(self):
        return len(self.entries)

    def clear(self):
        self.entries.clear()
