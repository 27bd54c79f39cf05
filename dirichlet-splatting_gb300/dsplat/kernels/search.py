"""Range gating, separated peaks and quasi-Newton steps of the spatial search (replaces
the reference's dsplat/kernels/search.py bindings of search.slang)."""

from __future__ import annotations

import ctypes
import math

import torch

from . import _lib
from ._lib import call, f32, ptr


def range_gate(points, positions, intervals, spacing, min_fraction):
    """Points whose spherical range bin lies in a marked interval at min_fraction of apertures."""
    points, positions = f32(points), f32(positions)
    intervals = intervals.to(torch.int32).contiguous()
    output = torch.empty(len(points), device=points.device, dtype=torch.int32)
    required = math.ceil(min_fraction * len(positions) - 1e-7)
    call(
        "dsg_range_gate", ptr(points), len(points), ptr(positions) if len(positions) else None,
        len(positions), ptr(intervals) if intervals.numel() else None, intervals.shape[1],
        float(spacing), required, ptr(output), _lib.stream(points.device),
    )  # fmt: skip
    return output.bool()


def peaks(scores, centers, count, separation):
    """Greedy best-first indices at least separation apart."""
    scores = scores.float().contiguous()
    centers = f32(centers)
    wanted = min(count, len(scores))
    output = torch.empty((wanted,), device=centers.device, dtype=torch.int32)
    order = torch.sort(scores, descending=True, stable=True).indices.to(torch.int32)
    call(
        "dsg_peaks", ptr(scores) if len(scores) else None, ptr(order) if len(order) else None,
        ptr(centers) if len(centers) else None, len(scores), centers.shape[1], wanted,
        float(separation), ptr(output), _lib.stream(centers.device),
    )  # fmt: skip
    return output[output >= 0].long()


def distinct(scores, points, occupied, period, separation, width):
    """Best-scoring candidates that collide neither with occupied points nor with each other."""
    scores = scores.float().contiguous()
    points, occupied = f32(points), f32(occupied)
    order = torch.sort(scores, descending=True, stable=True).indices.to(torch.int32)
    output = torch.empty((max(width, 1),), device=points.device, dtype=torch.int32)
    kept = torch.zeros((1,), device=points.device, dtype=torch.int32)
    per = None if period is None else torch.as_tensor(period, dtype=torch.float32, device=points.device)
    call(
        "dsg_distinct", ptr(scores) if len(scores) else None, ptr(order) if len(order) else None,
        ptr(points) if len(points) else None, len(scores), points.shape[1],
        ptr(occupied) if len(occupied) else None, len(occupied), ptr(per), float(separation),
        int(width), ptr(output), ptr(kept), _lib.stream(points.device),
    )  # fmt: skip
    return output[: int(kept.item())].long()


def direction(inverse, gradient, normals, mask, radius):
    """Quasi-Newton descent per candidate: tangent to unit normals, inside the trust radius."""
    count, width = gradient.shape
    gradient = f32(gradient)
    output = torch.empty_like(gradient)
    call(
        "dsg_direction", ptr(f32(inverse)), ptr(gradient), ptr(f32(normals)), ptr(f32(mask)),
        count, width, float(radius), ptr(output), _lib.stream(gradient.device),
    )  # fmt: skip
    return output


def trial(centers, normals, direction, controls, fraction):
    """Step fraction along direction, clamped to the box and renormalized; frozen axes kept.

    controls rows: per-coordinate scale, trainable mask, lower and upper bounds.
    """
    count, width = direction.shape
    centers, normals = f32(centers), f32(normals)
    out_centers, out_normals = torch.empty_like(centers), torch.empty_like(normals)
    call(
        "dsg_trial", ptr(centers), ptr(normals), ptr(f32(direction)), ptr(f32(controls)), count,
        width, float(fraction), ptr(out_centers), ptr(out_normals), _lib.stream(centers.device),
    )  # fmt: skip
    return out_centers, out_normals


def trials(centers, normals, direction, controls, fractions):
    """trial for every fraction in one launch: centers and normals [len(fractions), count, 3]."""
    count, width = direction.shape
    centers, normals = f32(centers), f32(normals)
    shape = (len(fractions), count, 3)
    out_centers, out_normals = centers.new_empty(shape), normals.new_empty(shape)
    values = (ctypes.c_float * len(fractions))(*fractions)
    call(
        "dsg_trials", ptr(centers), ptr(normals), ptr(f32(direction)), ptr(f32(controls)), count, width,
        ctypes.addressof(values), len(fractions), ptr(out_centers), ptr(out_normals), _lib.stream(centers.device),
    )  # fmt: skip
    return out_centers, out_normals


def ascent_spec(specs):
    """DsgAscentSpec of a search's ParameterConfigs (centers, and normals when present)."""
    groups = list(specs.values())
    spec = _lib.AscentSpec()
    spec.width = 3 * len(groups)
    for k, group in enumerate(groups):
        spec.normalize[k] = int(group.normalize)
        spec.scale[k] = float(group.scale)
        flags = group.trainable if isinstance(group.trainable, tuple) else (group.trainable,) * 3
        for j in range(3):
            spec.mask[3 * k + j] = 1.0 if flags[j] else 0.0
    return spec


def ascent_partition(corr, norm, areas, power, real_mode, value, trial_centers, trial_normals, stuck=None):
    """Full-step improvement flags, slots of the stable pending-first partition, the pending
    count (device) and the batch rows of the smaller fractions at those slots; candidates
    flagged in stuck (uint8) are never pending."""
    fractions, count = trial_centers.shape[:2]
    device = value.device
    areas = f32(areas)
    improved = torch.empty(count, dtype=torch.uint8, device=device)
    position = torch.empty(count, dtype=torch.int32, device=device)
    pending = torch.empty(1, dtype=torch.int32, device=device)
    rows = max(fractions - 1, 0) * count
    batch_centers = torch.empty((rows, 3), dtype=torch.float32, device=device)
    batch_normals = torch.empty((rows, 3), dtype=torch.float32, device=device)
    call(
        "dsg_ascent_partition", ptr(torch.view_as_real(corr)), ptr(norm), ptr(areas), ptr(power), int(real_mode),
        ptr(value), count, ptr(trial_centers), ptr(trial_normals), fractions, ptr(stuck), ptr(improved),
        ptr(position), ptr(pending), ptr(batch_centers) if rows else None, ptr(batch_normals) if rows else None,
        _lib.stream(device),
    )  # fmt: skip
    return improved, position, pending, batch_centers, batch_normals


def ascent_select(corr, norm, areas, power, real_mode, value, improved, position, trial_centers, trial_normals,
                  centers, normals, move_normals, stuck=None):  # fmt: skip
    """New centers and normals (the first improving fraction, else unchanged) and accepted."""
    fractions, count = trial_centers.shape[:2]
    areas = f32(areas)
    new_centers, new_normals = torch.empty_like(centers), torch.empty_like(normals)
    accepted = torch.empty(count, dtype=torch.uint8, device=value.device)
    call(
        "dsg_ascent_select", None if corr is None else ptr(torch.view_as_real(corr)), ptr(norm), ptr(areas),
        ptr(power), int(real_mode), ptr(value), count, ptr(improved), ptr(position), ptr(trial_centers),
        ptr(trial_normals), fractions, ptr(stuck), ptr(centers), ptr(normals), int(move_normals), ptr(new_centers),
        ptr(new_normals), ptr(accepted), _lib.stream(value.device),
    )  # fmt: skip
    return new_centers, new_normals, accepted


def ascent_update(spec, corr, norm, dcorr, dnorm, areas, power, real_mode, new_centers, new_normals, accepted,
                  centers, normals, value, gradient, inverse):  # fmt: skip
    """Value, ascent gradient, BFGS inverse and parameters of every candidate, in place."""
    areas = f32(areas)
    call(
        "dsg_ascent_update", ctypes.byref(spec), ptr(torch.view_as_real(corr)), ptr(norm),
        ptr(torch.view_as_real(dcorr)), ptr(dnorm), ptr(areas), ptr(power), int(real_mode), len(value),
        ptr(new_centers), ptr(new_normals), ptr(accepted), ptr(centers), ptr(normals), ptr(value), ptr(gradient),
        ptr(inverse), _lib.stream(value.device),
    )  # fmt: skip


def backward_elimination(inverse, rhs, count, limited=None, limit=0):
    """Removal order of backward elimination from the float64 inverse (dsg_backward_elimination)."""
    n = len(inverse)
    device = inverse.device
    removed = torch.empty((count,), dtype=torch.long, device=device)
    if count == 0:
        return removed
    complex_mode = inverse.is_complex()
    dtype = torch.complex128 if complex_mode else torch.float64
    w = inverse.to(dtype).contiguous()
    q = rhs.to(dtype).contiguous()
    lim = None if limited is None else limited.to(torch.uint8).contiguous()
    nbytes = _lib.query("dsg_elimination_workspace_bytes", n, count, int(complex_mode))
    work, nbytes = _lib.workspace(nbytes, device)
    call(
        "dsg_backward_elimination", ptr(w), ptr(q), n, count, None if lim is None else ptr(lim),
        int(limit), int(complex_mode), ptr(work), nbytes, ptr(removed), _lib.stream(device),
    )  # fmt: skip
    return removed


def triangular_inverse(factor):
    """L^-1 of a lower-triangular float64 / complex128 Cholesky factor (dsg_triangular_inverse).

    Recursive halving, [[A, 0], [B, C]]^-1 = [[A^-1, 0], [-C^-1 B A^-1, C^-1]]: every
    64-row diagonal block is inverted by one forward-substitution launch, each off-diagonal
    block is two triangular products (cuBLAS trmm).
    """
    complex_mode = factor.is_complex()
    x = factor.to(torch.complex128 if complex_mode else torch.float64).clone().contiguous()
    n = len(x)
    if n == 0:
        return x
    info = torch.zeros((1,), dtype=torch.int32, device=x.device)
    nbytes = _lib.query("dsg_triangular_inverse_workspace_bytes", n, int(complex_mode))
    work, nbytes = _lib.workspace(nbytes, x.device)
    call("dsg_triangular_inverse", ptr(x), n, int(complex_mode), ptr(work), nbytes, ptr(info), _lib.stream(x.device))
    return x


def backward_elimination_factor(factor_inverse, rhs, count, limited=None, limit=0):
    """backward_elimination from X = L^-1 (the inverse being X^H X), dsg_backward_elimination_factor."""
    n = len(factor_inverse)
    device = factor_inverse.device
    removed = torch.empty((count,), dtype=torch.long, device=device)
    if count == 0:
        return removed
    complex_mode = factor_inverse.is_complex()
    dtype = torch.complex128 if complex_mode else torch.float64
    x = factor_inverse.to(dtype).contiguous()
    q = rhs.to(dtype).contiguous()
    lim = None if limited is None else limited.to(torch.uint8).contiguous()
    nbytes = _lib.query("dsg_elimination_workspace_bytes", n, count, int(complex_mode))
    work, nbytes = _lib.workspace(nbytes, device)
    call(
        "dsg_backward_elimination_factor", ptr(x), ptr(q), n, count, None if lim is None else ptr(lim),
        int(limit), int(complex_mode), ptr(work), nbytes, ptr(removed), _lib.stream(device),
    )  # fmt: skip
    return removed
