"""Residual certificate: normalized correlations, candidate grids, peaks and ascent.

The certificate of an atom a against a residual r is |s|^2 / (|a|^2 |r|^2) with
s = a^H r (complex coefficients) or Re(a^H r) (signed-real); it ranks insertions.
Semantics of the reference's dsplat/certificate.py:11-201. The correlations are the
aperture-reduced CUDA kernels; the per-candidate algebra stays in float64 so the 1e-60
norm floor is representable; peaks, ascent directions and trial steps are the search
kernels. The batched ascent (no device reads inside the loop, CUDA-graph replay) is
dsplat.ascent.
"""

from __future__ import annotations

from dataclasses import dataclass
from math import ceil

import torch

from .kernels import search

NORM_FLOOR = 1e-60
PEAK_POOL = 64  # candidates kept per wanted peak before suppression


def certificate(model, params, residual, mode, *, gradient=False, normals=False, active=None):
    """Squared normalized certificate per atom, optionally with its explicit gradient.

    The gradient is by centers, and by normals too when normals is set. active (count
    tensor, period) lets the model skip atoms whose index mod period is not below count;
    their values are then meaningless and the caller masks them.
    """
    if gradient:
        corr, norm, dcorr, dnorm = model.correlate_gradient(params, residual, include_normals=normals)
    elif active is not None:
        corr, norm = model.correlate(params, residual, active=active)
    else:
        corr, norm = model.correlate(params, residual)
    energy = residual.abs().square().sum().double().clamp(min=1e-30)
    c = corr.to(torch.complex128)
    n = norm.double().clamp(min=NORM_FLOOR)
    projected = c.real if mode == "real" else c
    value = projected.abs().square() / (n * energy)
    if not gradient:
        return value.float()
    dc = dcorr.to(torch.complex128)
    dn = torch.where((n > NORM_FLOOR)[:, None], dnorm.double(), 0.0)
    if mode == "real":
        dnum = 2 * projected[:, None] * dc.real
    else:
        dnum = 2 * (c.conj()[:, None] * dc).real
    slope = (dnum - (value * energy)[:, None] * dn) / (n * energy)[:, None]
    return value.float(), slope.float()


@dataclass(frozen=True)
class CertificateSearchConfig:
    peaks: int = 1024  # separated coarse peaks refined per search
    separation: float = 0.0005  # center units, for coarse peak selection
    iterations: int = 40  # quasi-Newton ascent steps
    trust_radius: float = 1.0  # times each parameter's scale
    backtracks: int = 8


def candidate_grid(lower, upper, spacing, device="cuda"):
    """Regular grid [points, D] spanning both box corners, pitch at most spacing."""
    axes = [torch.linspace(lo, hi, 1 + ceil((hi - lo) / spacing), device=device)
            for lo, hi in zip(lower, upper, strict=True)]  # fmt: skip
    return torch.cartesian_prod(*axes).reshape(-1, len(axes))


def select_peaks(scores, centers, count, separation):
    """Greedy nonmaximum suppression: best-first indices at least separation apart.

    With many more scores than wanted peaks, the suppression first runs on the
    PEAK_POOL * count best (every score at or above that level, in index order); if that
    pool already yields every wanted peak, nothing below it could change the result.
    """
    if separation == 0:
        best = scores.argsort(descending=True, stable=True)[:count]
        return best[torch.isfinite(scores[best])]
    wanted = min(count, len(scores))
    if len(scores) > PEAK_POOL * wanted:
        level = scores.topk(PEAK_POOL * wanted).values[-1]
        pool = torch.nonzero(scores >= level).flatten()
        chosen = search.peaks(scores[pool], centers[pool], wanted, separation)
        if len(chosen) == wanted:
            return pool[chosen]
    return search.peaks(scores, centers, count, separation)


def fibonacci_sphere(count, device="cuda"):
    """Nearly uniform unit vectors [count, 3] on the golden-angle spiral."""
    index = torch.arange(count, device=device, dtype=torch.float32)
    z = 1 - (2 * index + 1) / count
    turn = index * (torch.pi * (3 - 5**0.5))
    ring = (1 - z * z).sqrt()
    return torch.stack((ring * torch.cos(turn), ring * torch.sin(turn), z), -1)


@torch.no_grad()
def orient_candidates(model, params, residual, count, mode, table=None, chunk=1 << 21, fused=False):
    """Each position with the best normal among its own and a count-normal sphere bank.

    Returns the candidates with the chosen normals and their squared certificates. One
    launch scores a chunk of positions against all 1 + count normals; fused (models with
    orient_best) also selects the best normal in that launch instead of writing every
    normal's scores for the selection here.
    """
    centers = params["centers"]
    bank = fibonacci_sphere(count, centers.device)
    energy = residual.abs().square().sum().double().clamp(min=1e-30)
    best_scores, best_normals = [], []
    for start in range(0, len(centers), chunk):
        part = {key: value[start : start + chunk] for key, value in params.items()}
        if fused:
            which, top = model.orient_best(part, residual, bank, energy, mode == "real", table)
            own = part["normals"]
            if len(bank):
                own = torch.where((which == 0)[:, None], own, bank[(which - 1).clamp(min=0)])
            best_normals.append(own)
            best_scores.append(top)
            continue
        corr, norm = model.correlate_orientations(part, residual, bank, table)
        c = corr.to(torch.complex128)
        projected = c.real if mode == "real" else c
        value = projected.abs().square() / (norm.double().clamp(min=NORM_FLOOR) * energy)
        top, which = value.max(1)
        choices = torch.cat((part["normals"][:, None, :], bank[None].expand(len(which), -1, -1)), 1)
        best_normals.append(choices[torch.arange(len(which), device=which.device), which])
        best_scores.append(top.float())
    return {**params, "normals": torch.cat(best_normals)}, torch.cat(best_scores)


def _controls(reference, center_spec, normal_spec, masks):
    """[4, 6] rows per coordinate (centers xyz, normals xyz): step scale, trainable mask,
    lower bound, upper bound; the layout the direction and trial kernels read."""
    table = reference.new_zeros((4, 6))
    table[0, :3] = center_spec.scale
    table[1, :3] = masks["centers"]
    table[2, :3] = reference.new_tensor(-torch.inf if center_spec.lower is None else center_spec.lower)
    table[3, :3] = reference.new_tensor(torch.inf if center_spec.upper is None else center_spec.upper)
    if normal_spec is not None:
        table[0, 3:] = normal_spec.scale
        table[1, 3:] = 1
    return table


def _scaled_descent(params, gradient, masks, specs):
    """The negative certificate gradient in each field's tangent, masked and scaled units."""
    pieces = []
    for i, (key, spec) in enumerate(specs.items()):
        part = spec.tangent(gradient[:, 3 * i : 3 * i + 3], params[key])
        pieces.append(part * masks[key] * spec.scale)
    return -torch.cat(pieces, -1)


@torch.no_grad()
def search_certificate(
    model, residual, candidates, center_spec, config, mode, *, normal_spec=None,
    initial_scores=None, full_model=None, full_residual=None, batched=False,
):  # fmt: skip
    """Refine separated peaks in xyz (and unit normals) by quasi-Newton ascent.

    Every candidate backtracks on its own inside the parameter constraints. The coarse
    peaks stay beside the refined ones, and all are reranked on full_model and
    full_residual when given. Returns (parameters, scores), best first. batched runs
    dsplat.ascent (same result up to the rounding of the correlation sums).
    """
    from . import ascent

    anchor = candidates["centers"]
    feasible = dict(candidates, centers=center_spec.project(anchor, anchor))
    specs = {"centers": center_spec}
    if normal_spec is not None:
        specs["normals"] = normal_spec
        feasible["normals"] = normal_spec.project(candidates["normals"], candidates["normals"])
    masks = {key: spec.mask(feasible[key]) for key, spec in specs.items()}
    controls = _controls(anchor, center_spec, normal_spec, masks)

    def score(params, gradient=False, active=None):
        return certificate(model, params, residual, mode, gradient=gradient, normals="normals" in specs,
                           active=active)  # fmt: skip

    coarse_scores = score(feasible) if initial_scores is None else initial_scores
    ids = select_peaks(coarse_scores, feasible["centers"], config.peaks, config.separation)
    coarse = {key: value[ids] for key, value in feasible.items()}
    params = {key: value.clone() for key, value in coarse.items()}
    value, grad = score(params, True)
    grad = _scaled_descent(params, grad, masks, specs)
    count, width = grad.shape
    eye = torch.eye(width, device=anchor.device).expand(count, width, width)
    inverse = eye.clone()
    fractions = [0.5**k for k in range(config.backtracks)]
    if batched and anchor.is_cuda:
        params, value, grad, inverse = ascent.run(model, residual, controls, masks, specs, config, mode, fractions,
                                                  eye, params, value, grad, inverse)  # fmt: skip
    else:
        for _ in range(config.iterations):
            direction = search.direction(inverse, grad, params["normals"], controls[1], config.trust_radius)
            start = {key: v.clone() for key, v in params.items()}
            moved = torch.zeros(count, dtype=torch.bool, device=anchor.device)
            for fraction in fractions:
                centers, normals = search.trial(start["centers"], start["normals"], direction, controls, fraction)
                open_ids = torch.nonzero(~moved).flatten()
                trial = {key: v[open_ids] for key, v in dict(start, centers=centers, normals=normals).items()}
                gained = score(trial)
                take = torch.zeros_like(moved)
                take[open_ids] = torch.isfinite(gained) & (gained > value[open_ids])
                if "centers" in specs:
                    params["centers"][take] = centers[take]
                if "normals" in specs:
                    params["normals"][take] = normals[take]
                moved |= take
                if bool(moved.all()):
                    break
            if not bool(moved.any()):
                break
            new_value, new_grad = score(params, True)
            new_grad = _scaled_descent(params, new_grad, masks, specs)
            inverse = ascent._bfgs_update(inverse, start, params, grad, new_grad, moved, specs, eye)
            value, grad = new_value, new_grad
    merged = {key: torch.cat((coarse[key], params[key])) for key in params}
    if full_model is None:
        scores = torch.cat((coarse_scores[ids], value))
    else:
        scores = certificate(full_model, merged, full_residual, mode)
    order = scores.argsort(descending=True, stable=True)
    return {key: v[order] for key, v in merged.items()}, scores[order]
