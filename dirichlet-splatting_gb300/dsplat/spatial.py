"""Spatial candidate search: hierarchical 3-D grids and continuous certificate refinement.

Every step, before replacement, builds a fresh candidate pool inside the box of the
centers' bounds:

  1. a coarse grid over the box (finer and shifted after failed steps), range-gated by
     the measured profiles, plus the peaks kept from the previous step;
  2. per finer level, a cube of offsets around every separated peak of the last level;
  3. quasi-Newton certificate ascent of the separated peaks on an aperture subset, then
     of the best few on every aperture.

Positions are scored with their best normal from a sphere bank (FFT-interpolated range
table, one CUDA launch per chunk) when normals are trainable; fields the search does not
move copy slot 0. Semantics of the reference's dsplat/spatial.py:26-178.
"""

from __future__ import annotations

from dataclasses import dataclass, field, replace
from math import ceil, prod

import torch

from .certificate import (
    CertificateSearchConfig,
    candidate_grid,
    certificate,
    orient_candidates,
    search_certificate,
    select_peaks,
)
from .tracing import stage

GRID_SHIFT = (0.37, 0.61, 0.23)  # cell fractions of the coarse grid's shift after failures
REFINE_SEED = 1000003  # seed offset of the refinement's aperture subset


@dataclass(frozen=True)
class SpatialSearchConfig:
    coarse_spacing: float = 0.002  # metres
    # (radius, pitch) of each finer level; every level samples a cube around every peak.
    levels: tuple[tuple[float, float], ...] = ((0.002, 0.0005), (0.0005, 0.000125))
    proposal_apertures: int = 384  # apertures scoring the grids
    refine_apertures: int = 768  # apertures of the first continuous refinement
    max_candidates: int = 2_000_000  # points per grid level
    range_power: float = 0.03  # range-gate threshold relative to each profile's peak
    range_margin_cells: float = 1.5  # range-gate dilation in range resolutions
    range_fraction: float = 0.7  # share of apertures a candidate must hit
    ungated_after: int = 2  # failed steps after which the gate is dropped
    normal_candidates: int = 24  # sphere-bank normals tried per position; 0 keeps the slot's
    joint_normals: bool = True  # refine trainable normals with the positions
    fft_oversample: int = 8  # FFT-interpolated proposal scores; 0 is exact
    cache_peaks: int = 256  # peak locations carried to the next step
    full_peaks: int = 64  # peaks refined again on every aperture
    full_iterations: int = 8
    continuous: CertificateSearchConfig = field(default_factory=CertificateSearchConfig)


def _grid_size(lower, upper, pitch):
    """Points candidate_grid(lower, upper, pitch) would make."""
    return prod(1 + ceil(float(hi - lo) / pitch) for lo, hi in zip(lower, upper, strict=True))


def _coarsened(lower, upper, pitch, budget):
    """pitch grown by 10 % steps until the grid fits in budget points."""
    while _grid_size(lower, upper, pitch) > budget:
        pitch *= 1.1
    return pitch


def _take(atoms, index):
    return {key: value[index] for key, value in atoms.items()}


def _free_axes(spec, width=3):
    """Per-axis trainable flags of a field, on the host."""
    flags = spec.trainable
    return [bool(f) for f in flags] if isinstance(flags, (tuple, list)) else [bool(flags)] * width


class _Proposer:
    """One step's search: the sampled apertures, the residual, and how positions are scored."""

    def __init__(self, state, config, search):
        self.state, self.config, self.search = state, config, search
        self.spec = state.parameters["centers"]
        self.normal_spec = state.parameters["normals"]
        normals_free = self.normal_spec.any_free
        self.refine_normals = self.normal_spec if normals_free and search.joint_normals else None
        self.mode = config.coefficients
        self.residual = state.target - state.prediction
        self.ids, self.model = state.model.sample_apertures(search.proposal_apertures,
                                                            config.seed + state.iteration)  # fmt: skip
        self.sub_residual = self.residual[self.ids]
        self.banked = normals_free and search.normal_candidates > 0
        oversample = search.fft_oversample
        self.table = self.model.range_table(self.sub_residual, oversample) if self.banked and oversample else None

    def atoms(self, points, normals=None):
        """Feasible atoms at points (fields copied from slot 0), optionally with normals."""
        size = len(points)
        result = {key: value[:1].expand(size, *value.shape[1:]).clone() for key, value in self.state.params.items()}
        result["centers"] = self.spec.project(points, result["centers"])
        if normals is not None:
            result["normals"] = self.normal_spec.project(normals, result["normals"])
        return result

    def score(self, candidates):
        """Certificates on the sampled apertures; with a bank, the candidates take their best normal."""
        if not self.banked:
            return certificate(self.model, candidates, self.sub_residual, self.mode)
        fused = getattr(self.config, "batched", False) and hasattr(self.model, "orient_best")
        oriented, scores = orient_candidates(self.model, candidates, self.sub_residual, self.search.normal_candidates,
                                             self.mode, self.table, fused=fused)  # fmt: skip
        candidates["normals"] = oriented["normals"]
        return scores

    def coarse_candidates(self):
        """Range-gated coarse grid over the box plus the cached peaks of the last step."""
        state, search, spec = self.state, self.search, self.spec
        centers = state.params["centers"]
        failures = state.search_failures
        free = _free_axes(spec)
        box = torch.stack((centers.new_tensor(spec.lower).expand(3), centers.new_tensor(spec.upper).expand(3)))
        pinned = [axis for axis in range(3) if not free[axis]]
        if pinned:
            box[:, pinned] = centers[0, pinned]
        lower, upper = box.tolist()
        spacing = _coarsened(lower, upper, search.coarse_spacing / (1 + min(failures, 2)), search.max_candidates)
        points = candidate_grid(lower, upper, spacing, device=centers.device)
        if failures:
            shift = points.new_tensor(GRID_SHIFT) * (spacing * ((failures % 3) + 1) / 3)
            points = spec.project(points + shift, points)
        if failures < search.ungated_after:
            loosen = 1 + failures
            hit = self.model.range_gate(points, state.target[self.ids], relative_power=search.range_power / loosen,
                                        margin_cells=search.range_margin_cells * loosen,
                                        min_fraction=search.range_fraction)  # fmt: skip
            if bool(hit.any()):  # an empty gate never stops the search
                points = points[hit]
        carried = 0
        if state.peak_cache is not None:
            carried = min(len(state.peak_cache["centers"]), search.max_candidates - len(points))
            points = torch.cat((points, state.peak_cache["centers"][:carried]))
        candidates = self.atoms(points)
        if carried:
            tail = candidates["normals"][-carried:]
            candidates["normals"][-carried:] = self.normal_spec.project(state.peak_cache["normals"][:carried], tail)
        return candidates

    def level_candidates(self, peaks, radius, pitch):
        """A cube of offsets (radius, pitch) around each peak; frozen axes get no offsets."""
        free = _free_axes(self.spec)
        low = [-radius if f else 0.0 for f in free]
        high = [radius if f else 0.0 for f in free]
        pitch = _coarsened(low, high, pitch, self.search.max_candidates)
        offsets = candidate_grid(low, high, pitch, device=peaks["centers"].device)
        # the best-ranked peaks keep priority inside the per-level budget
        peaks = {key: value[: max(1, self.search.max_candidates // len(offsets))] for key, value in peaks.items()}
        points = (peaks["centers"][:, None, :] + offsets[None]).reshape(-1, 3)
        return self.atoms(points, peaks["normals"].repeat_interleave(len(offsets), dim=0))


@torch.no_grad()
def propose(state, config, search):
    """Refined candidates, their scores best first, and the peaks kept for the next step.

    After failed steps (state.search_failures) the coarse grid gets finer and shifts by a
    fraction of a cell, more peaks are kept and the range gate loosens.
    """
    finder = _Proposer(state, config, search)
    ascent_config = search.continuous
    wanted = min(ascent_config.peaks * (1 + state.search_failures), 4 * ascent_config.peaks)
    separation = ascent_config.separation
    batched = getattr(config, "batched", False)

    candidates = finder.coarse_candidates()
    with stage("propose.coarse"):
        scores = finder.score(candidates)
        kept = select_peaks(scores, candidates["centers"], wanted, separation)
        candidates = _take(candidates, kept)
    for radius, pitch in search.levels:
        candidates = finder.level_candidates(candidates, radius, pitch)
        with stage("propose.level"):
            scores = finder.score(candidates)
            kept = select_peaks(scores, candidates["centers"], wanted, min(separation, radius / 2))
            candidates = _take(candidates, kept)
    # FFT-interpolated scores only propose; exact ones may seed the refinement
    model, residual = finder.model, finder.sub_residual
    initial = scores[kept] if finder.table is None else None
    if search.refine_apertures > search.proposal_apertures:
        refine_ids, model = state.model.sample_apertures(search.refine_apertures,
                                                         config.seed + state.iteration + REFINE_SEED)  # fmt: skip
        residual, initial = finder.residual[refine_ids], None
    with stage("propose.refine"):
        params, scores = search_certificate(
            model, residual, candidates, finder.spec, replace(ascent_config, peaks=wanted, separation=0),
            finder.mode, normal_spec=finder.refine_normals, initial_scores=initial, full_model=state.model,
            full_residual=finder.residual, batched=batched)  # fmt: skip
    if search.full_iterations:
        finalists = select_peaks(scores, params["centers"], search.full_peaks, min(separation, finder.spec.scale / 2))
        with stage("propose.full"):
            refined, refined_scores = search_certificate(
                state.model, finder.residual, _take(params, finalists), finder.spec,
                replace(ascent_config, peaks=search.full_peaks, iterations=search.full_iterations, separation=0),
                finder.mode, normal_spec=finder.refine_normals, initial_scores=scores[finalists],
                batched=batched)  # fmt: skip
        # the screened finalists stay in the pool beside the fully refined ones
        scores = torch.cat((refined_scores, scores))
        order = scores.argsort(descending=True, stable=True)
        params = {key: torch.cat((value, params[key]))[order] for key, value in refined.items()}
        scores = scores[order]
    if not search.cache_peaks:
        return params, scores, None
    cache = select_peaks(scores, params["centers"], search.cache_peaks, separation)
    return params, scores, {key: value[cache].clone() for key, value in params.items()}
