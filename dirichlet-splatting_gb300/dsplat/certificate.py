"""Residual certificate: normalized correlations, candidate grids, peaks and refinement.

The certificate of an atom a against a residual r is |s|^2 / (|a|^2 |r|^2) with
s = a^H r (complex coefficients) or Re(a^H r) (signed-real). It ranks insertions.
Behaviour follows the reference's dsplat/certificate.py:11-201; the correlations run
on the aperture-reduced CUDA kernels and the peaks / quasi-Newton steps on the
search kernels.
"""

from __future__ import annotations

from dataclasses import dataclass, replace
from math import ceil

import torch

from .kernels import search
from .tracing import stage


def certificate(model, params, residual, mode, *, gradient=False, normals=False, active=None):
    """Squared normalized certificate per atom, optionally with its explicit gradient.

    The gradient is by centers, and by normals too when normals is set. The small
    per-candidate algebra runs in double so the 1e-60 norm floor is representable.
    active (count tensor, period) lets the model skip atoms whose index mod period is not
    below count; their values are then meaningless and must be masked by the caller.
    """
    if gradient:
        c, n, dc, dn = model.correlate_gradient(params, residual, include_normals=normals)
    elif active is not None:
        c, n = model.correlate(params, residual, active=active)
    else:
        c, n = model.correlate(params, residual)
    c, n = c.to(torch.complex128), n.double().clamp(min=1e-60)
    power = residual.abs().square().sum().double().clamp(min=1e-30)
    s = c.real if mode == "real" else c
    value = s.abs().square() / n / power
    if not gradient:
        return value.float()
    dc = dc.to(torch.complex128)
    dn = torch.where((n > 1e-60)[:, None], dn.double(), 0)
    ds = 2 * s[:, None] * dc.real if mode == "real" else 2 * (c.conj()[:, None] * dc).real
    return value.float(), ((ds - value[:, None] * power * dn) / n[:, None] / power).float()


@dataclass(frozen=True)
class CertificateSearchConfig:
    peaks: int = 1024  # separated coarse peaks refined per search
    separation: float = 0.0005  # center units, for coarse peak selection
    iterations: int = 40  # quasi-Newton ascent steps
    trust_radius: float = 1.0  # times each parameter's scale
    backtracks: int = 8


def candidate_grid(lower, upper, spacing, device="cuda"):
    """Regular grid including both box corners; the actual pitch never exceeds spacing."""
    axes = [
        torch.linspace(a, b, 1 + ceil((b - a) / spacing), device=device)
        for a, b in zip(lower, upper, strict=True)
    ]
    return torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, len(axes))


PEAK_POOL = 64  # candidates kept per wanted peak before suppression


def select_peaks(scores, centers, count, separation):
    """Greedy nonmaximum suppression: best-first indices at least separation apart."""
    if separation == 0:
        order = scores.argsort(descending=True, stable=True)[:count]
        return order[torch.isfinite(scores[order])]
    wanted = min(count, len(scores))
    if len(scores) > PEAK_POOL * wanted:
        # Everything at or above the pool's score level is decided before anything below
        # it, so when the pool already yields every peak the rest cannot change the
        # result; index order inside the pool keeps the tie-breaking.
        level = scores.topk(PEAK_POOL * wanted).values[-1]
        pool = (scores >= level).nonzero().flatten()
        chosen = search.peaks(scores[pool], centers[pool], wanted, separation)
        if len(chosen) == wanted:
            return pool[chosen]
    return search.peaks(scores, centers, count, separation)


def fibonacci_sphere(count, device="cuda"):
    """Nearly uniform unit vectors [count, 3] on the golden-angle spiral."""
    j = torch.arange(count, device=device, dtype=torch.float32)
    z = 1 - 2 * (j + 0.5) / count
    angle = j * (torch.pi * (3 - 5**0.5))
    radius = (1 - z.square()).sqrt()
    return torch.stack((radius * angle.cos(), radius * angle.sin(), z), -1)


@torch.no_grad()
def orient_candidates(model, params, residual, count, mode, table=None, chunk=1 << 21):
    """Give every position the best normal among its own and a count-normal sphere bank.

    Returns the candidates with the chosen normals and their squared certificates.
    chunk only bounds the [chunk, 1 + count] score buffers; one launch scores a chunk.
    """
    centers = params["centers"]
    bank = fibonacci_sphere(count, centers.device)
    power = residual.abs().square().sum().double().clamp(min=1e-30)
    scores, normals = [], []
    for start in range(0, len(centers), chunk):
        block = {key: value[start : start + chunk] for key, value in params.items()}
        c, n = model.correlate_orientations(block, residual, bank, table)
        c, n = c.to(torch.complex128), n.double()
        s = c.real if mode == "real" else c
        best, ids = (s.abs().square() / n.clamp(min=1e-60) / power).max(1)
        normal = block["normals"].clone()
        from_bank = ids > 0
        normal[from_bank] = bank[ids[from_bank] - 1]
        scores.append(best.float())
        normals.append(normal)
    return {**params, "normals": torch.cat(normals)}, torch.cat(scores)


def _controls(reference, center_spec, normal_spec, masks):
    """[4, 6] per-coordinate rows: step scale, trainable mask, lower and upper bound."""
    controls = reference.new_zeros((4, 6))
    controls[0, :3] = center_spec.scale
    controls[1, :3] = masks["centers"]
    lower = -torch.inf if center_spec.lower is None else center_spec.lower
    upper = torch.inf if center_spec.upper is None else center_spec.upper
    controls[2, :3] = reference.new_tensor(lower)
    controls[3, :3] = reference.new_tensor(upper)
    if normal_spec is not None:
        controls[0, 3:] = normal_spec.scale
        controls[1, 3:] = 1
    return controls


@torch.no_grad()
def search_certificate(
    model, residual, candidates, center_spec, config, mode, *, normal_spec=None,
    initial_scores=None, full_model=None, full_residual=None, batched=False,
):  # fmt: skip
    """Refine separated peaks in xyz (and unit normals) by batched quasi-Newton ascent.

    Every candidate backtracks on its own inside the parameter constraints. The coarse
    peaks stay beside the refined ones, and all are reranked on full_model and
    full_residual when given. Returns parameters and scores, best first.

    batched scores all backtracking fractions of an iteration in one correlation launch
    and never reads a device value inside the ascent loop: each candidate still takes
    the largest fraction that raises its score, and an iteration without any accepted
    step changes nothing, so the result is the sequential search's up to the rounding
    of the correlation sums.
    """
    reference = candidates["centers"]
    feasible = dict(candidates, centers=center_spec.project(reference, reference))
    specs = {"centers": center_spec}
    if normal_spec is not None:
        specs["normals"] = normal_spec
        feasible["normals"] = normal_spec.project(candidates["normals"], candidates["normals"])
    masks = {key: spec.mask(feasible[key]) for key, spec in specs.items()}
    controls = _controls(reference, center_spec, normal_spec, masks)

    ascent, score = _closures(model, residual, masks, specs, mode)
    coarse_scores = score(feasible) if initial_scores is None else initial_scores
    ids = select_peaks(coarse_scores, feasible["centers"], config.peaks, config.separation)
    coarse = {key: value[ids] for key, value in feasible.items()}
    params = {key: value.clone() for key, value in coarse.items()}
    value, grad = score(params, True)
    grad = ascent(params, grad)
    count, dim = grad.shape
    eye = torch.eye(dim, device=reference.device).expand(count, dim, dim)
    inverse = eye.clone()
    fractions = [0.5**backtrack for backtrack in range(config.backtracks)]

    iterate = _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye)
    if batched and config.iterations > 1 and reference.is_cuda:
        params, value, grad, inverse = _cached_ascent(model, residual, controls, masks, specs, config, mode,
                                                      fractions, eye, params, value, grad, inverse)  # fmt: skip
    else:
        for _ in range(config.iterations):
            if batched:
                params, value, grad, inverse = iterate(params, value, grad, inverse)
                continue
            direction = search.direction(inverse, grad, params["normals"], controls[1],
                                         config.trust_radius)  # fmt: skip
            old = {key: v.clone() for key, v in params.items()}
            accepted = torch.zeros(count, dtype=torch.bool, device=reference.device)
            for fraction in fractions:
                centers, normals = search.trial(old["centers"], old["normals"], direction, controls,
                                                fraction)  # fmt: skip
                trial = dict(old, centers=centers, normals=normals)
                pending = torch.where(~accepted)[0]
                trial_value = score({key: v[pending] for key, v in trial.items()})
                keep = torch.zeros_like(accepted)
                keep[pending] = torch.isfinite(trial_value) & (trial_value > value[pending])
                for key in specs:
                    params[key][keep] = trial[key][keep]
                accepted |= keep
                if accepted.all():
                    break
            if not accepted.any():
                break
            new_value, new_grad = score(params, True)
            new_grad = ascent(params, new_grad)
            inverse = _bfgs_update(inverse, old, params, grad, new_grad, accepted, specs, eye)
            value, grad = new_value, new_grad
    combined = {key: torch.cat((coarse[key], params[key])) for key in params}
    if full_model is None:
        scores = torch.cat((coarse_scores[ids], value))
    else:
        scores = certificate(full_model, combined, full_residual, mode)
    order = scores.argsort(descending=True, stable=True)
    return {key: v[order] for key, v in combined.items()}, scores[order]


def _closures(model, residual, masks, specs, mode):
    """ascent(params, gradient) and score(params, gradient, active) of one search."""

    def ascent(params, gradient):
        """Negative gradient in scaled tangent coordinates (the quantity minimized)."""
        parts = [
            spec.tangent(gradient[:, 3 * i : 3 * i + 3], params[key]) * masks[key] * spec.scale
            for i, (key, spec) in enumerate(specs.items())
        ]
        return -torch.cat(parts, -1)

    def score(params, gradient=False, active=None):
        return certificate(model, params, residual, mode, gradient=gradient,
                           normals="normals" in specs, active=active)  # fmt: skip

    return ascent, score


def _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye):
    """One batched ascent iteration (params, value, grad, inverse) -> the same, all on device."""
    ascent, score = _closures(model, residual, masks, specs, mode)

    def iterate(params, value, grad, inverse):
        direction = search.direction(inverse, grad, params["normals"], controls[1], config.trust_radius)
        old = {key: v.clone() for key, v in params.items()}
        params, accepted = _backtrack_batched(old, direction, controls, fractions, value, specs, score)
        new_value, new_grad = score(params, True)
        new_grad = ascent(params, new_grad)
        inverse = _bfgs_update(inverse, old, params, grad, new_grad, accepted, specs, eye)
        return params, new_value, new_grad, inverse

    return iterate


_ASCENTS: dict = {}


def _cached_ascent(model, residual, controls, masks, specs, config, mode, fractions, eye, params, value, grad,
                   inverse):  # fmt: skip
    """The batched ascent replayed from a CUDA graph kept across searches of the same shape.

    The graph reads the apertures, the residual, the controls and masks from static
    buffers that every search refills, so a later search of the same shapes and settings
    replays all its iterations without capturing again. Models without a scan of
    apertures capture per search (_graphed_ascent).
    """
    from .kernels import _lib

    if _fusable(model, params, fractions):
        return _fused_ascent(model, residual, controls, specs, config, mode, fractions, params, value, grad, inverse)
    if not hasattr(model, "scan") or not hasattr(model, "fresnel_n"):
        iterate = _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye)
        return _graphed_ascent(iterate, config.iterations, params, value, grad, inverse)
    positions = model.scan.scan_positions_m
    key = (repr(model.scan.fmcw_config), model.fresnel_n, tuple(positions.shape), tuple(residual.shape),
           residual.dtype, mode, repr(specs), repr(config), tuple(fractions), positions.device,
           tuple((k, tuple(v.shape), v.dtype) for k, v in params.items()), tuple(grad.shape))  # fmt: skip
    entry = _ASCENTS.get(key)
    if entry is None:
        # everything the graph reads by address stays referenced by the cache entry
        static_inputs = {"positions": positions.clone(), "residual": residual.clone(), "controls": controls.clone(),
                         "masks": {k: m.clone() for k, m in masks.items()}, "eye": eye.clone()}  # fmt: skip
        static_model = replace(model, scan=replace(model.scan, scan_positions_m=static_inputs["positions"]))
        iterate = _iteration(static_model, static_inputs["residual"], static_inputs["controls"],
                             static_inputs["masks"], specs, config, mode, fractions, static_inputs["eye"])  # fmt: skip
        params, value, grad, inverse = _graphed_ascent(iterate, config.iterations, params, value, grad, inverse,
                                                       keep=(key, static_inputs))  # fmt: skip
        return params, value, grad, inverse
    graph, static_inputs, static, per_replay = entry
    static_inputs["positions"].copy_(positions)
    static_inputs["residual"].copy_(residual)
    static_inputs["controls"].copy_(controls)
    for k, m in masks.items():
        static_inputs["masks"][k].copy_(m)
    for k, v in params.items():
        static[0][k].copy_(v)
    static[1].copy_(value)
    static[2].copy_(grad)
    static[3].copy_(inverse)
    with stage("ascent.replay"):
        for _ in range(config.iterations):
            graph.replay()
    _lib.REPLAYED_LAUNCHES += per_replay * config.iterations
    return ({k: v.clone() for k, v in static[0].items()}, static[1].clone(), static[2].clone(),
            static[3].clone())  # fmt: skip


def _fusable(model, params, fractions):
    """Surfel models on CUDA whose candidates carry centers, normals and areas only."""
    return (hasattr(model, "scan") and hasattr(model, "sensor") and hasattr(model, "fresnel_n")
            and sorted(params) == ["areas", "centers", "normals"] and params["centers"].is_cuda
            and 1 <= len(fractions) <= 16)  # fmt: skip


def _fused_iteration(model, residual, power, controls, specs, config, mode, fractions):
    """One batched ascent iteration on the state buffers, in place, in eight launches.

    The correlations run on the surfel kernels without the area factors, which the
    fused kernels apply: dsg_trials, the full-step correlation, dsg_ascent_partition,
    the active-set correlation of the smaller fractions, dsg_ascent_select, the
    correlation gradient and dsg_ascent_update replace the PyTorch algebra of
    _iteration (the same arithmetic, up to the order of float sums).
    """
    from .kernels import surfel as kernel

    chirp, positions = model.sensor
    shaped = residual.reshape(model.shape)
    real_mode = mode == "real"
    spec = search.ascent_spec(specs)
    move_normals = "normals" in specs

    def iterate(params, value, grad, inverse):
        centers, normals, areas = params["centers"], params["normals"], params["areas"]
        direction = search.direction(inverse, grad, normals, controls[1], config.trust_radius)
        trial_centers, trial_normals = search.trials(centers, normals, direction, controls, fractions)
        corr, norm = kernel.correlate(chirp, positions, trial_centers[0], trial_normals[0], shaped, model.fresnel_n)
        improved, position, pending, batch_centers, batch_normals = search.ascent_partition(
            corr, norm, areas, power, real_mode, value, trial_centers, trial_normals)  # fmt: skip
        corr2 = norm2 = None
        if len(fractions) > 1:
            corr2, norm2 = kernel.correlate(chirp, positions, batch_centers, batch_normals, shaped, model.fresnel_n,
                                            active=(pending, len(value)))  # fmt: skip
        new_centers, new_normals, accepted = search.ascent_select(
            corr2, norm2, areas, power, real_mode, value, improved, position, trial_centers, trial_normals,
            centers, normals, move_normals)  # fmt: skip
        c, n, dc, dn = kernel.correlate_gradient(chirp, positions, new_centers, new_normals, shaped, model.fresnel_n,
                                                 move_normals)  # fmt: skip
        search.ascent_update(spec, c, n, dc, dn, areas, power, real_mode, new_centers, new_normals, accepted,
                             centers, normals, value, grad, inverse)  # fmt: skip

    return iterate


def _fused_ascent(model, residual, controls, specs, config, mode, fractions, params, value, grad, inverse):
    """The fused batched ascent, its graph kept across searches of the same shapes.

    The state (parameters, value, gradient, inverse) and the inputs (apertures, residual
    and its power, controls) live in static buffers that every search refills; the first
    search runs one iteration eagerly (the capture's warm-up), captures the next and
    replays it, a later one replays every iteration.
    """
    from .kernels import _lib

    positions = model.scan.scan_positions_m
    key = ("fused", repr(model.scan.fmcw_config), model.fresnel_n, tuple(positions.shape), tuple(residual.shape),
           residual.dtype, mode, repr(specs), repr(config), tuple(fractions), positions.device,
           tuple((k, tuple(v.shape)) for k, v in params.items()), tuple(grad.shape))  # fmt: skip
    power = residual.abs().square().sum().double().clamp(min=1e-30).reshape(1)
    entry = _ASCENTS.get(key)
    if entry is not None:
        graph, inputs, state, per_replay = entry
        inputs["positions"].copy_(positions)
        inputs["residual"].copy_(residual)
        inputs["controls"].copy_(controls)
        inputs["power"].copy_(power)
        for k, v in params.items():
            state[0][k].copy_(v)
        state[1].copy_(value)
        state[2].copy_(grad)
        state[3].copy_(inverse)
        with stage("ascent.replay"):
            for _ in range(config.iterations):
                graph.replay()
        _lib.REPLAYED_LAUNCHES += per_replay * config.iterations
    else:
        inputs = {"positions": positions.clone(), "residual": residual.contiguous().clone(),
                  "controls": controls.contiguous().clone(), "power": power.clone()}  # fmt: skip
        state = ({k: v.float().contiguous().clone() for k, v in params.items()}, value.float().contiguous().clone(),
                 grad.float().contiguous().clone(), inverse.float().contiguous().clone())  # fmt: skip
        static_model = replace(model, scan=replace(model.scan, scan_positions_m=inputs["positions"]))
        iterate = _fused_iteration(static_model, inputs["residual"], inputs["power"], inputs["controls"], specs,
                                   config, mode, fractions)  # fmt: skip
        device = value.device
        side = torch.cuda.Stream(device)
        side.wait_stream(torch.cuda.current_stream(device))
        timers, _lib.TIMERS = _lib.TIMERS, None  # events cannot be timed inside a graph
        try:
            with stage("ascent.capture"):
                with torch.cuda.stream(side):
                    iterate(*state)
                torch.cuda.current_stream(device).wait_stream(side)
                graph = torch.cuda.CUDAGraph()
                before = _lib.library().dsg_launch_count()
                with torch.cuda.graph(graph):
                    iterate(*state)
                per_replay = _lib.library().dsg_launch_count() - before
            with stage("ascent.replay"):
                for _ in range(config.iterations - 1):
                    graph.replay()
            _lib.REPLAYED_LAUNCHES += per_replay * (config.iterations - 1)
            _ASCENTS[key] = (graph, inputs, state, per_replay)
        finally:
            _lib.TIMERS = timers
    return ({k: v.clone() for k, v in state[0].items()}, state[1].clone(), state[2].clone(), state[3].clone())


def _bfgs_update(inverse, old, params, grad, new_grad, accepted, specs, eye):
    """Damped BFGS update of each candidate's inverse Hessian (skipped where invalid)."""
    step = torch.cat([(params[k] - old[k]) / spec.scale for k, spec in specs.items()], -1)
    change = new_grad - grad
    sy = (step * change).sum(-1)
    valid = accepted & (sy > 1e-8 * step.norm(dim=-1) * change.norm(dim=-1)) & (sy > 1e-20)
    rho = torch.where(valid, 1 / sy.clamp(min=1e-30), 0)
    left = eye - rho[:, None, None] * step[:, :, None] * change[:, None, :]
    updated = left @ inverse @ left.transpose(-1, -2) + rho[:, None, None] * step[:, :, None] * step[:, None, :]
    return torch.where(valid[:, None, None], updated, inverse)


def _graphed_ascent(iterate, iterations, params, value, grad, inverse, keep=None):
    """Run the batched ascent: one eager iteration, then the rest replayed from a CUDA graph.

    The iteration reads and writes only device tensors of fixed shapes, so the graph
    captured from the second iteration replays every later one; the eager first
    iteration doubles as the warm-up that capture needs.
    """
    from .kernels import _lib

    device = value.device
    side = torch.cuda.Stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    timers, _lib.TIMERS = _lib.TIMERS, None  # events cannot be timed inside a graph
    try:
        with stage("ascent.capture"):
            with torch.cuda.stream(side):
                state = iterate(params, value, grad, inverse)
                static = ({k: v.clone() for k, v in state[0].items()}, state[1].clone(), state[2].clone(),
                          state[3].clone())  # fmt: skip
            torch.cuda.current_stream(device).wait_stream(side)
            graph = torch.cuda.CUDAGraph()
            before = _lib.library().dsg_launch_count()
            with torch.cuda.graph(graph):
                out = iterate(*static)
                for key, v in out[0].items():
                    static[0][key].copy_(v)
                static[1].copy_(out[1])
                static[2].copy_(out[2])
                static[3].copy_(out[3])
            per_replay = _lib.library().dsg_launch_count() - before
        with stage("ascent.replay"):
            for _ in range(iterations - 1):
                graph.replay()
        _lib.REPLAYED_LAUNCHES += per_replay * (iterations - 1)
        if keep is not None:  # (key, static inputs) of _cached_ascent
            _ASCENTS[keep[0]] = (graph, keep[1], static, per_replay)
    finally:
        _lib.TIMERS = timers
    return ({k: v.clone() for k, v in static[0].items()}, static[1].clone(), static[2].clone(),
            static[3].clone())  # fmt: skip


def _backtrack_batched(old, direction, controls, fractions, value, specs, score):
    """All backtracking trials of one iteration scored without host synchronization.

    Each candidate takes the first (largest) fraction whose finite score exceeds value.
    The full step is scored for every candidate; the smaller fractions only for those the
    full step did not improve, compacted to the front of each fraction's block, with the
    pending count kept on the device (score(batch, active=(count, period)) skips the rest).
    """
    count = len(old["centers"])
    trials = [search.trial(old["centers"], old["normals"], direction, controls, f) for f in fractions]
    centers = torch.stack([c for c, _ in trials])  # [B, count, 3]
    normals = torch.stack([n for _, n in trials])
    first_values = score(dict(old, centers=centers[0], normals=normals[0]))
    improve_first = torch.isfinite(first_values) & (first_values > value)
    rows = torch.arange(count, device=value.device)
    if len(fractions) > 1:
        # Pending candidates first (stable), the improved ones after them.
        order = torch.argsort(improve_first.to(torch.int8), stable=True)
        pending = (~improve_first).sum().to(torch.int32).reshape(1)
        rest = len(fractions) - 1
        batch = {key: v[order].repeat(rest, *([1] * (v.ndim - 1))) for key, v in old.items()}
        batch["centers"] = centers[1:, order].reshape(-1, 3)
        batch["normals"] = normals[1:, order].reshape(-1, 3)
        values = score(batch, active=(pending, count)).reshape(rest, count)
        live = rows[None] < pending  # compacted position holds a pending candidate
        improve = torch.isfinite(values) & (values > value[order][None]) & live
        later = improve.any(0)
        step = improve.to(torch.int8).argmax(0) + 1  # fraction index, compacted order
        accepted_later = torch.zeros_like(improve_first).scatter(0, order, later)
        fraction_later = torch.zeros_like(rows).scatter(0, order, step)
    else:
        accepted_later = torch.zeros_like(improve_first)
        fraction_later = torch.zeros_like(rows)
    accepted = improve_first | accepted_later
    first = torch.where(improve_first, 0, fraction_later)
    params = dict(old)
    keep = accepted[:, None]
    if "centers" in specs:
        params["centers"] = torch.where(keep, centers[first, rows], old["centers"])
    if "normals" in specs:
        params["normals"] = torch.where(keep, normals[first, rows], old["normals"])
    return params, accepted
