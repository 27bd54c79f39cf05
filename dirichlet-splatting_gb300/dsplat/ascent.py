"""Batched certificate ascent on the device: every candidate's backtracking in one pass.

The sequential ascent (certificate.search_certificate) scores each backtracking fraction
of each iteration and reads back which candidates improved. Here one iteration never
reads a device value: the full step is scored for every candidate and the smaller
fractions only for those it did not improve (compacted to the front, the pending count
kept on the device), each candidate takes the largest improving fraction, and an
iteration without accepted steps changes nothing. The result equals the sequential
search up to the rounding of the correlation sums, so the iterations replay from a CUDA
graph: for surfel models the iteration is eight fused launches (dsg_trials, the
full-step correlation, dsg_ascent_partition, the active-set correlation,
dsg_ascent_select, the correlation gradient, dsg_ascent_update), and the graph is kept
across searches of the same shapes with its inputs in static buffers.
"""

from __future__ import annotations

from dataclasses import replace

import torch

from .graphs import GraphCache, recording, side_stream
from .kernels import search
from .tracing import stage


def _closures(model, residual, masks, specs, mode):
    """descent(params, gradient) and score(params, gradient, active) of one search."""
    from .certificate import _scaled_descent, certificate

    def descent(params, gradient):
        return _scaled_descent(params, gradient, masks, specs)

    def score(params, gradient=False, active=None):
        return certificate(model, params, residual, mode, gradient=gradient, normals="normals" in specs,
                           active=active)  # fmt: skip

    return descent, score


def run(model, residual, controls, masks, specs, config, mode, fractions, eye, params, value, grad, inverse):
    """config.iterations batched ascent iterations; replayed from a CUDA graph when several."""
    if config.iterations > 1:
        return _cached_ascent(model, residual, controls, masks, specs, config, mode, fractions, eye, params, value,
                              grad, inverse)  # fmt: skip
    iterate = _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye)
    for _ in range(config.iterations):
        params, value, grad, inverse = iterate(params, value, grad, inverse)
    return params, value, grad, inverse


def _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye):
    """One batched ascent iteration (params, value, grad, inverse) -> the same, all on device."""
    descent, score = _closures(model, residual, masks, specs, mode)

    def iterate(params, value, grad, inverse):
        direction = search.direction(inverse, grad, params["normals"], controls[1], config.trust_radius)
        old = {key: v.clone() for key, v in params.items()}
        params, accepted = _backtrack_batched(old, direction, controls, fractions, value, specs, score)
        new_value, new_grad = score(params, True)
        new_grad = descent(params, new_grad)
        inverse = _bfgs_update(inverse, old, params, grad, new_grad, accepted, specs, eye)
        return params, new_value, new_grad, inverse

    return iterate


_ASCENTS = GraphCache()


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


def _fused_iteration(model, residual, power, controls, specs, config, mode, fractions, tables=None):
    """One batched ascent iteration on the state buffers, in place, in eight launches.

    The correlations run on the surfel kernels without the area factors, which the
    fused kernels apply: dsg_trials, the full-step correlation, dsg_ascent_partition,
    the active-set correlation of the smaller fractions, dsg_ascent_select, the
    correlation gradient and dsg_ascent_update replace the PyTorch algebra of
    _iteration (the same arithmetic, up to the order of float sums).

    stuck (uint8 per candidate) marks candidates that rejected every fraction: their state
    did not change, so the same trials fail again in every later iteration (the kernels
    are deterministic); they are kept out of the active set, which removes most of the
    backtracking work once the ascent converges, without changing any result.

    tables (kernel.residual_tables of the residual, with derivative) lets the three
    correlations of every iteration read the residual's interpolation tables instead of
    rebuilding them from the residual (bitwise the same results).
    """
    from .kernels import surfel as kernel

    chirp, positions = model.sensor
    shaped = residual.reshape(model.shape)
    real_mode = mode == "real"
    spec = search.ascent_spec(specs)
    move_normals = "normals" in specs

    def iterate(params, value, grad, inverse, stuck):
        centers, normals, areas = params["centers"], params["normals"], params["areas"]
        direction = search.direction(inverse, grad, normals, controls[1], config.trust_radius)
        trial_centers, trial_normals = search.trials(centers, normals, direction, controls, fractions)
        corr, norm = kernel.correlate(chirp, positions, trial_centers[0], trial_normals[0], shaped, model.fresnel_n,
                                      tables=tables)  # fmt: skip
        improved, position, pending, batch_centers, batch_normals = search.ascent_partition(
            corr, norm, areas, power, real_mode, value, trial_centers, trial_normals, stuck)  # fmt: skip
        corr2 = norm2 = None
        if len(fractions) > 1:
            corr2, norm2 = kernel.correlate(chirp, positions, batch_centers, batch_normals, shaped, model.fresnel_n,
                                            active=(pending, len(value)), tables=tables)  # fmt: skip
        new_centers, new_normals, accepted = search.ascent_select(
            corr2, norm2, areas, power, real_mode, value, improved, position, trial_centers, trial_normals,
            centers, normals, move_normals, stuck)  # fmt: skip
        stuck.copy_(stuck | (accepted == 0).to(torch.uint8))
        c, n, dc, dn = kernel.correlate_gradient(chirp, positions, new_centers, new_normals, shaped, model.fresnel_n,
                                                 move_normals, tables=tables)  # fmt: skip
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
    from .kernels import surfel as kernel

    positions = model.scan.scan_positions_m
    tabled = kernel.interpolated()
    key = ("fused", tabled, repr(model.scan.fmcw_config), model.fresnel_n, tuple(positions.shape), tuple(residual.shape),
           residual.dtype, mode, repr(specs), repr(config), tuple(fractions), positions.device,
           tuple((k, tuple(v.shape)) for k, v in params.items()), tuple(grad.shape))  # fmt: skip
    power = residual.abs().square().sum().double().clamp(min=1e-30).reshape(1)
    entry = _ASCENTS.get(key)
    if entry is not None:
        graph, inputs, state, per_replay = entry
        inputs["positions"].copy_(positions)
        inputs["residual"].copy_(residual)
        if tabled:  # once per search: every iteration's correlations read them
            kernel.residual_tables(model.sensor[0], inputs["residual"].reshape(model.shape), out=inputs["tables"])
        inputs["controls"].copy_(controls)
        inputs["power"].copy_(power)
        inputs["stuck"].zero_()
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
                  "controls": controls.contiguous().clone(), "power": power.clone(),
                  "stuck": torch.zeros(len(value), dtype=torch.uint8, device=value.device)}  # fmt: skip
        inputs["tables"] = (kernel.residual_tables(model.sensor[0], inputs["residual"].reshape(model.shape))
                            if tabled else None)  # fmt: skip
        state = ({k: v.float().contiguous().clone() for k, v in params.items()}, value.float().contiguous().clone(),
                 grad.float().contiguous().clone(), inverse.float().contiguous().clone())  # fmt: skip
        static_model = replace(model, scan=replace(model.scan, scan_positions_m=inputs["positions"]))
        iterate = _fused_iteration(static_model, inputs["residual"], inputs["power"], inputs["controls"], specs,
                                   config, mode, fractions, inputs["tables"])  # fmt: skip
        device = value.device
        side = side_stream(device)
        side.wait_stream(torch.cuda.current_stream(device))
        timers, _lib.TIMERS = _lib.TIMERS, None  # events cannot be timed inside a graph
        try:
            with stage("ascent.capture"):
                with torch.cuda.stream(side):
                    iterate(*state, inputs["stuck"])
                torch.cuda.current_stream(device).wait_stream(side)
                graph = torch.cuda.CUDAGraph()
                before = _lib.library().dsg_launch_count()
                with recording(graph):
                    iterate(*state, inputs["stuck"])
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
    """Quasi-Newton update of each candidate's inverse Hessian H [C, D, D] after a step.

    With s the accepted step in scaled units, y the gradient change and rho = 1 / s.y,
    H+ = H - rho (s (Hy)^T + (Hy) s^T) + (rho^2 y.Hy + rho) s s^T (the BFGS inverse
    update written out for a symmetric H). A candidate keeps H when it did not move or
    when s.y is not safely positive (curvature condition).
    """
    del eye  # the expanded form needs no identity
    s = torch.cat([(params[key] - old[key]) / spec.scale for key, spec in specs.items()], -1)
    y = new_grad - grad
    sy = (s * y).sum(-1)
    usable = accepted & (sy > 1e-8 * s.norm(dim=-1) * y.norm(dim=-1)) & (sy > 1e-20)
    rho = torch.where(usable, 1 / sy.clamp(min=1e-30), 0)[:, None, None]
    hy = (inverse @ y[:, :, None])[..., 0]
    yhy = (y * hy).sum(-1)[:, None, None]
    outer_s = s[:, :, None] * s[:, None, :]
    mixed = s[:, :, None] * hy[:, None, :]
    updated = inverse - rho * (mixed + mixed.transpose(-1, -2)) + (rho * rho * yhy + rho) * outer_s
    return torch.where(usable[:, None, None], updated, inverse)


def _graphed_ascent(iterate, iterations, params, value, grad, inverse, keep=None):
    """Run the batched ascent: one eager iteration, then the rest replayed from a CUDA graph.

    The iteration reads and writes only device tensors of fixed shapes, so the graph
    captured from the second iteration replays every later one; the eager first
    iteration doubles as the warm-up that capture needs.
    """
    from .kernels import _lib

    device = value.device
    side = side_stream(device)
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
            with recording(graph):
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
