"""Reference semantics of the search kernels and the energy reduction (oracle; test-only).

Restates dsplat/kernels/search.slang:7-109 and dsplat/kernels/reduce.slang:3-21 as
plain float64 / integer PyTorch on the CPU.
"""

from __future__ import annotations

import math

import torch


def range_gate(points, positions, intervals, spacing, min_fraction):
    """Boolean [count]: round-half-even range bin inside a marked interval at enough apertures."""
    required = math.ceil(min_fraction * len(positions) - 1e-7)
    x = (points.double()[:, None] - positions.double()[None]).norm(dim=-1) / spacing
    k = torch.round(x).long()  # torch.round is half-to-even
    bins = intervals.shape[1]
    valid = (k >= 0) & (k < bins)
    hit = torch.zeros_like(valid)
    idx = torch.arange(len(positions))[None].expand_as(k)
    hit[valid] = intervals.bool()[idx[valid], k[valid]]
    return hit.sum(1) >= required


def peaks(scores, centers, count, separation):
    """Greedy best-first indices (ties to the lowest index) at least separation apart."""
    scores = scores.double().clone()
    centers = centers.double()
    chosen = []
    for _ in range(min(count, len(scores))):
        finite = torch.isfinite(scores)
        if not finite.any():
            break
        best = scores.masked_fill(~finite, -math.inf)
        top = best.max()
        index = int(torch.nonzero(best == top)[0])
        chosen.append(index)
        near = (centers - centers[index]).square().sum(1) < separation * separation
        scores[near] = -math.inf
        scores[index] = -math.inf
    return torch.tensor(chosen, dtype=torch.long)


def direction(inverse, gradient, normals, mask, radius):
    d = -(inverse.double() @ gradient.double()[..., None])[..., 0]
    g = gradient.double()
    descent = (d * g).sum(-1, keepdim=True)
    d = torch.where(descent >= 0, -g, d) * mask.double()[: g.shape[1]]
    if g.shape[1] == 6:
        n = normals.double()
        d[:, 3:] -= (d[:, 3:] * n).sum(-1, keepdim=True) * n
    scale = (radius / d.norm(dim=-1, keepdim=True).clamp(min=1e-30)).clamp(max=1)
    return d * scale


def trial(centers, normals, direction, controls, fraction):
    width = direction.shape[1]
    c = centers.double() + fraction * controls[0, :3].double() * direction[:, :3].double()
    c = torch.minimum(torch.maximum(c, controls[2, :3].double()), controls[3, :3].double())
    c = torch.where(controls[1, :3] > 0, c, centers.double())
    if width == 6:
        n = normals.double() + fraction * controls[0, 3:].double() * direction[:, 3:].double()
        n = n / n.norm(dim=-1, keepdim=True)
    else:
        n = normals.double()
    return c, n


def energy(value, reference):
    return (value.to(torch.complex128) - reference.to(torch.complex128)).abs().square().sum()
