"""DSFW: replace support, refine geometry, accept on the full objective, repeat.

A step is three stages over an immutable state (tensors are shared between states and
never written in place, so any earlier state can be stepped again):

  propose   a fresh candidate pool from the spatial search (with a SpatialSearchConfig),
            else the fixed pool given to initialize;
  replace   merged (pool many candidates, keep the budget's best) or utility (one slot);
  slide     a geometry step (joint Gauss-Newton or dense LM), skipped with a doubling
            back-off while it gains less than lm_gain_ratio times the replacement.

Defaults are the fast 3-D configuration: signed-real coefficients, merged replacement of
up to 1024 pooled candidates, joint Gauss-Newton on 1024 apertures. Semantics of the
reference's dsplat/dsfw.py:20-174. Two fields are this build's: DSFWConfig.gram selects
the arithmetic of the streamed real Gram ("fp32": SSYRK, the reference's; "bf16x3":
split-BF16x3 on the tcgen05 tensor cores), DSFWConfig.batched the device-resident
execution of the search and replacement loops.
"""

from __future__ import annotations

from dataclasses import dataclass, replace

import torch

from .parameters import ParameterConfig
from .normal import PROJECTIONS
from .refinement import dense_slide, joint_slide, trainable
from .replacement import merge_support, replace_one
from .spatial import propose
from .tracing import stage
from .varpro import varpro

LM_WAIT_LIMIT = 8  # longest run of skipped geometry steps; see DSFWConfig.lm_gain_ratio
SCREEN_SEED = 2000003  # seed offset of the screening aperture subset


@dataclass(frozen=True)
class DSFWConfig:
    iterations: int = 80
    ridge: float = 0.0  # on the mean-square data term
    coefficients: str = "real"  # "real" (signed) or "complex"
    replacement: str = "merged"  # "merged" or "utility" (one slot per step)
    batch: int = 1024  # merged: candidates pooled with the support per step
    min_separation: float = 0.0  # replacement candidates' distance from the support
    lm_solver: str = "joint_cg"  # "joint_cg" or "dense"
    lm_steps: int = 1
    # Skip the geometry step while it lowers the objective by less than this fraction of
    # the replacement's gain: for one step, then two, doubling up to LM_WAIT_LIMIT, until
    # it pays again. Zero runs it every step.
    lm_gain_ratio: float = 1.0
    lm_rows: int = 4096  # dense: sampled observation rows
    # Seeded apertures of the joint_cg proposal system and of the subset check that
    # rejects clearly worse proposals before the full evaluation; 0, at least the
    # aperture count, or a SpectralModel uses everything.
    joint_apertures: int = 1024
    screen_apertures: int = 1024
    cg_iterations: int = 16
    cg_tolerance: float = 1e-3
    cg_probes: int = 2
    damping: float = 1e-3
    trust_radius: float = 1.5  # dimensionless; times each ParameterConfig.scale
    row_chunk: int = 65536
    dictionary_elements: int = 32_000_000  # observations x atoms per streamed block
    seed: int = 0
    gram: str = "fp32"  # "fp32" or "bf16x3": arithmetic of the real Gram products
    batched: bool = False  # device-resident search / replacement loops (same results up to rounding)

    @property
    def real(self):
        """Signed-real coefficients; a misspelt mode raises KeyError."""
        return {"real": True, "complex": False}[self.coefficients]


@dataclass(frozen=True)
class DSFWState:
    model: object
    target: torch.Tensor
    params: dict
    candidates: dict  # the replacement pool without a spatial search
    parameters: dict  # name -> ParameterConfig
    coefficients: torch.Tensor
    prediction: torch.Tensor
    objective: float
    gram: torch.Tensor  # Re(A^H A) / M for real coefficients, A^H A / M otherwise
    rhs: torch.Tensor
    power: float  # mean |target|^2
    iteration: int = 0
    history: tuple = ()
    peak_cache: dict | None = None  # spatial-search peaks carried to the next step
    search_failures: int = 0
    lm_skip: int = 0  # steps left before the geometry step runs again
    lm_wait: int = 0  # length of the current run of skipped steps


def _logged(state, config, **extra):
    """state with one history entry appended: iteration, objective, NMSE (+ extra)."""
    penalty = config.ridge * float(state.coefficients.abs().square().sum()) if config.ridge else 0.0
    # a zero target fits exactly with zero coefficients; its NMSE is then 0
    nmse = (state.objective - penalty) / max(state.power, torch.finfo(torch.float32).tiny)
    entry = {"iteration": state.iteration, "objective": state.objective, "nmse": nmse, **extra}
    return replace(state, history=state.history + (entry,))


def _backoff(wait, poor):
    """Length of the next run of skipped geometry steps after a slide that paid (or not)."""
    return min(LM_WAIT_LIMIT, max(1, 2 * wait)) if poor else 0


@torch.no_grad()
def initialize(model, target, params, config, *, candidates=None, parameters=None):
    """Project params onto their constraints and fit the coefficients.

    candidates (default: params) are the replacement pool without a spatial search;
    fields they omit copy slot 0 (merged) or the replaced slot (utility). Fields without a
    ParameterConfig stay fixed.
    """
    given = parameters or {}
    specs = {key: given.get(key, ParameterConfig(trainable=False)) for key in params}
    start = {key: specs[key].project(value.detach().clone(), value.detach()) for key, value in params.items()}
    model = model.prepare(specs)
    if getattr(config, "gram", "fp32") == "bf16x3" and config.replacement == "merged":
        PROJECTIONS.track(model)  # the support's projected rows serve the next pool
    pool = start if candidates is None else {key: value.detach().clone() for key, value in candidates.items()}
    power = float(target.abs().square().mean())
    fit = varpro(model, start, target, config)
    return _logged(DSFWState(model, target, start, pool, specs, **fit._asdict(), power=power), config)


def _screen(state, config):
    """(model, target) of the seeded screening apertures, or None when screening is off."""
    if not 0 < config.screen_apertures < state.model.apertures:
        return None
    ids, model = state.model.sample_apertures(config.screen_apertures,
                                              config.seed + state.iteration + SCREEN_SEED)  # fmt: skip
    return model, state.target[ids]


@torch.no_grad()
def step(state, config, search=None):
    """One DSFW iteration; state.history[-1] describes it.

    With a SpatialSearchConfig the replacement pool is a fresh spatial search.
    """
    start_objective = state.objective
    pool, scores = state.candidates, None
    if search is not None:
        with stage("propose"):
            pool, scores, cache = propose(state, config, search)
        state = replace(state, peak_cache=cache)
    screen = _screen(state, config)
    merged = {"merged": True, "utility": False}[config.replacement]
    with stage("replace"):
        if merged:
            state, replaced = merge_support(state, config, pool, scores)
        else:
            state, replaced = replace_one(state, config, pool, screen)
    if search is not None:
        state = replace(state, search_failures=0 if replaced else state.search_failures + 1)
    replaced_objective = state.objective
    slides, skip, wait = 0, state.lm_skip, state.lm_wait
    if skip:
        skip -= 1
    elif trainable(state.params, state.parameters):
        slide = {"joint_cg": joint_slide, "dense": dense_slide}[config.lm_solver]
        with stage("slide"):
            state, slides = slide(state, config, screen)
        if config.lm_gain_ratio > 0:
            # the wait doubles while the slide keeps paying too little and ends as soon as
            # it pays again, so a late-stage slide is never starved
            gain = replaced_objective - state.objective
            wait = _backoff(wait, gain < config.lm_gain_ratio * (start_objective - replaced_objective))
            skip = wait
    state = replace(state, iteration=state.iteration + 1, lm_skip=skip, lm_wait=wait)
    return _logged(state, config, replaced=replaced, lm_accepted=slides)


def fit(model, target, params, config=None, search=None, *, candidates=None, parameters=None, callback=None):
    """initialize, then config.iterations steps; returns the final state.

    callback receives each step's history entry.
    """
    config = config or DSFWConfig()
    state = initialize(model, target, params, config, candidates=candidates, parameters=parameters)
    for _ in range(config.iterations):
        state = step(state, config, search)
        if callback is not None:
            callback(state.history[-1])
    return state
