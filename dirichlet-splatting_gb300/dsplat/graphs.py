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

from contextlib import contextmanager

import torch


@contextmanager
def recording(graph):
    """Capture the launches of the block into graph (a torch.cuda.CUDAGraph)."""
    current = torch.cuda.current_stream()
    side = torch.cuda.Stream(current.device)
    side.wait_stream(current)
    with torch.cuda.stream(side):
        graph.capture_begin()
        try:
            yield graph
        finally:
            graph.capture_end()
    current.wait_stream(side)
