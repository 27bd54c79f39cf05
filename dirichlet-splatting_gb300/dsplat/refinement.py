"""Local geometry refinement: dense reduced-VarPro LM and matrix-free joint Gauss-Newton.

Both propose a move of every trainable atom and keep it only when its refitted
objective is lower (varpro.accept), trying the full step, then shorter ones. Steps are
dimensionless; ParameterConfig.scale gives each field its unit. Semantics of the
reference's dsplat/refinement.py:20-227.

joint: the unknowns are every trainable geometry component and every coefficient,
scaled to unit steps; the Gauss-Newton matrix is never formed. A product with it is one
forward-mode JVP and one adjoint VJP on the CUDA kernels, its Jacobi diagonal is
estimated from Rademacher probes through the adjoint, and PCG (dsplat.linalg.pcg) runs
with a device-side stopping flag. dense: the coefficients are eliminated exactly on
sampled rows and the reduced Gauss-Newton system is formed and solved.
"""

from __future__ import annotations

import torch

from .linalg import pcg, solve
from .graphs import GraphCache, side_stream
from .tracing import stage
from .varpro import accept, fit_coefficients, screen_bar

BACKTRACK_JOINT = (1.0, 0.5, 0.25, 0.125)  # step fractions tried by the joint slide
BACKTRACK_DENSE = (1.0, 0.5, 0.25)  # step fractions tried by the dense slide


def trainable(params, specs):
    """[(key, spec)] of the fields with at least one free component, in specs order."""
    return [(key, spec) for key, spec in specs.items() if spec.any_free and key in params]


def probe_signs(shape, seed, device):
    """Successive Rademacher bit draws (0 / 1) of a device generator seeded with seed."""
    generator = torch.Generator(device=device).manual_seed(seed)
    while True:
        yield torch.randint(0, 2, shape, device=device, generator=generator)


def _as_matrix(value):
    return value[:, None] if value.ndim == 1 else value


def _free_width(spec, value):
    """Number of free components per atom, from the configuration (no device read)."""
    flags = spec.trainable
    if isinstance(flags, (tuple, list)):
        return sum(bool(flag) for flag in flags)
    return _as_matrix(value).shape[1] if flags else 0


# --- dense: reduced VarPro on sampled rows ---------------------------------------------------


@torch.no_grad()
def reduced_system(model, params, target, specs, config, rows):
    """Gauss-Newton matrix and gradient of the ridge-VarPro objective on the given rows.

    With every coefficient eliminated, the Jacobian of the residual is
    J = dA b + A db, db the exact differential of the least-squares coefficients
    (its right-hand side carries the dA^H r term); the unit-vector retraction and the
    parameter scales are chained in before the elimination.
    """
    a = model.design(params, rows)
    y = target.reshape(-1)[rows]
    m = len(a)
    gram, rhs = a.mH @ a / m, a.mH @ y / m
    b = fit_coefficients(gram, rhs, config)
    residual = a @ b.to(a.dtype) - y
    layout = trainable(params, specs)
    count = len(b)
    raw = model.jacobian(params, rows, torch.arange(count, device=a.device), [key for key, _ in layout])
    da = torch.cat([spec.differential(raw[key], params[key]) for key, spec in layout], -1)  # [m, S, D]
    width = da.shape[-1]
    j = (da * b[None, :, None]).reshape(m, count * width)
    cross = a.mH @ j / m
    # atom s's own columns also get sum_rows conj(dA[:, s, d]) r / m (the dA^H r term)
    own = torch.einsum("rsd,r->sd", da.conj(), residual) / m
    torch.diagonal(cross.view(count, count, width), dim1=0, dim2=1).add_(own.mT)
    h = gram.real if config.real else gram
    if config.ridge:
        h = h.clone()
        h.diagonal().add_(config.ridge)
    db = -solve(h, cross.real if config.real else cross, refined=getattr(config, "batched", False))
    reduced = j + a @ db.to(a.dtype)
    normal = (reduced.mH @ reduced / m + config.ridge * db.mH @ db).real
    gradient = (reduced.mH @ residual / m + config.ridge * db.mH @ b).real
    return normal, gradient


def _moved(state, layout, delta, fraction):
    """Parameters shifted by fraction * scale * delta on their free components, projected."""
    proposal = dict(state.params)
    column = 0
    for key, spec in layout:
        value = state.params[key]
        free = spec.mask(value)
        width = _free_width(spec, value)
        step = torch.zeros_like(_as_matrix(value))
        step[:, free] = delta[:, column : column + width] * (fraction * spec.scale)
        moved = _as_matrix(value) + step
        proposal[key] = spec.project(moved[:, 0] if value.ndim == 1 else moved, value)
        column += width
    return proposal


def dense_slide(state, config, screen=None):
    """Damped LM steps on lm_rows sampled rows with a trust radius per atom.

    Returns the state and the number of accepted steps.
    """
    layout = trainable(state.params, state.parameters)
    rows = state.model.sample_rows(config.lm_rows, config.seed + state.iteration, state.target.device)
    accepted = 0
    refined = getattr(config, "batched", False)
    for _ in range(config.lm_steps):
        normal, gradient = reduced_system(state.model, state.params, state.target, state.parameters, config, rows)
        diag = normal.diagonal()
        floor = diag.max() * 1e-6 + 1e-30
        damped = normal + config.damping * torch.diag(diag.clamp(min=floor))
        delta = solve(damped, -gradient, refined=refined).reshape(len(state.coefficients), -1)
        radius = delta.norm(dim=1, keepdim=True).clamp(min=1e-30)
        delta = delta * (config.trust_radius / radius).clamp(max=1)
        if not bool(torch.isfinite(delta).all()):
            break
        bar = screen_bar(screen, state.params, config)
        for fraction in BACKTRACK_DENSE:
            trial = accept(state, _moved(state, layout, delta, fraction), config, bar)
            if trial is not None:
                state, accepted = trial, accepted + 1
                break
        else:
            break
    return state, accepted


# --- joint: matrix-free Gauss-Newton over geometry and coefficients --------------------------


class _JointLayout:
    """Packing of the joint unknowns: per trainable field, count x free-width geometry
    entries (atom-major) in units of its scale; then the coefficients (re, im interleaved
    when complex) in units of coefficient_scale."""

    def __init__(self, params, specs, b, complex_mode):
        self.params, self.specs, self.b = params, specs, b
        self.complex = complex_mode
        self.count = len(b)
        self.sections = []  # (key, free component indices, slice)
        start = 0
        for key, spec in trainable(params, specs):
            free = spec.free_index(params[key])
            stop = start + self.count * _free_width(spec, params[key])
            self.sections.append((key, free, slice(start, stop)))
            start = stop
        self.geometry = start
        self.size = start + (2 if complex_mode else 1) * self.count
        amplitude = b.abs()
        self.amplitude = amplitude
        self.coefficient_scale = amplitude.clamp(min=amplitude.square().mean().sqrt() * 0.1 + 1e-20)

    def coefficient_entries(self, values):
        """Complex [count] per-coefficient values written into the packed coefficient slots."""
        return torch.view_as_real(values).reshape(-1) if self.complex else values.real

    def unpack(self, vector):
        """(tangent of every field, coefficient change) of a packed vector."""
        tangent = {key: torch.zeros_like(value) for key, value in self.params.items()}
        for key, free, section in self.sections:
            spec = self.specs[key]
            target = _as_matrix(tangent[key])
            target.index_copy_(1, free, vector[section].reshape(self.count, -1) * spec.scale)
            tangent[key] = spec.tangent(tangent[key], self.params[key])
        tail = vector[self.geometry :]
        if self.complex:
            return tangent, torch.complex(tail[0::2], tail[1::2]) * self.coefficient_scale
        return tangent, (tail * self.coefficient_scale).to(self.b.dtype)

    def pack_gradient(self, grads, coefficient):
        """Packed vector of field gradients (tangent, masked, scaled) and the coefficient one."""
        out = self.amplitude.new_zeros(self.size)
        for key, free, section in self.sections:
            spec = self.specs[key]
            along = _as_matrix(spec.tangent(grads[key], self.params[key]))
            out[section] = (along.index_select(1, free) * spec.scale).reshape(-1)
        out[self.geometry :] = self.coefficient_entries(coefficient * self.coefficient_scale)
        return out

    def step_lengths(self, tangent):
        """Per-atom length of a geometry tangent in units of each field's scale."""
        total = self.amplitude.new_zeros(self.count)
        for key, free, _ in self.sections:
            total += (_as_matrix(tangent[key]).index_select(1, free) / self.specs[key].scale).square().sum(1)
        return total.sqrt()


def joint_system(model, params, coefficients, target, specs, config, seed, pieces=None):
    """Scaled Gauss-Newton system of every trainable geometry component and coefficient.

    Returns (matvec, gradient, damped Jacobi diagonal, proposal(vector, fraction)).
    Products use the model's exact JVP and VJP; the Rademacher probes only estimate the
    diagonal. pieces, a dict, receives what matvec reads (b, layout, normalization, shift).
    """
    b = coefficients.to(target.dtype)
    layout = _JointLayout(params, specs, b, not config.real)
    power = target.abs().square().mean().clamp(min=1e-30)
    normalization = target.numel() * power
    ridge = config.ridge / power
    ridge_diagonal = layout.amplitude.new_zeros(layout.size)
    ridge_gradient = layout.amplitude.new_zeros(layout.size)
    scale = layout.coefficient_scale
    ridge_diagonal[layout.geometry :] = (ridge * scale.square()).repeat_interleave(2 if layout.complex else 1)
    ridge_gradient[layout.geometry :] = layout.coefficient_entries(b * (ridge * scale))

    def adjoint(upstream):
        grads, coefficient = model.vjp(params, b, upstream)
        return layout.pack_gradient(grads, coefficient)

    gradient = adjoint(model.render(params, b) - target) / normalization + ridge_gradient
    draws = probe_signs((*target.shape, 2), seed, b.device)
    diagonal = torch.zeros_like(gradient)
    for _ in range(config.cg_probes):
        probe = torch.view_as_complex((2 * next(draws) - 1).to(target.real.dtype))
        diagonal += adjoint(probe).square() / normalization
    diagonal = diagonal / config.cg_probes + ridge_diagonal
    diagonal = diagonal.clamp(min=diagonal.max().clamp(min=1e-30) * 1e-6)
    damping = config.damping * diagonal
    shift = ridge_diagonal + damping
    if pieces is not None:
        pieces.update(b=b, layout=layout, normalization=normalization, shift=shift)

    def matvec(vector):
        return adjoint(model.jvp(params, b, *layout.unpack(vector))) / normalization + shift * vector

    def proposal(vector, fraction):
        # one step scale for every atom keeps the joint direction; a unit normal's radial
        # part is a null direction and must not shrink the step
        tangent, _ = layout.unpack(vector)
        scale = (config.trust_radius / layout.step_lengths(tangent).max().clamp(min=1e-30)).clamp(max=1)
        return {key: specs[key].project(value + tangent[key] * (scale * fraction), value)
                for key, value in params.items()}  # fmt: skip

    return matvec, gradient, diagonal + damping, proposal


class _StaticJoint:
    """The joint system's matrix-vector product over fixed buffers (sensor positions of the
    aperture subset, parameters, coefficients, the layout's coefficient scale, the
    normalization and the damping shift), refilled per slide, so that one CUDA graph of the
    conjugate-gradient iteration serves every slide of the same shapes."""

    def __init__(self, model, params, specs, pieces, complex_mode):
        from dataclasses import replace

        self.positions = model.scan.scan_positions_m.clone()
        self.model = replace(model, scan=replace(model.scan, scan_positions_m=self.positions))
        self.params = {key: value.clone() for key, value in params.items()}
        self.b = pieces["b"].clone()
        self.layout = _JointLayout(self.params, specs, self.b, complex_mode)
        self.normalization = pieces["normalization"].clone()
        self.shift = pieces["shift"].clone()
        self.refill(model, params, pieces)

    def refill(self, model, params, pieces):
        self.positions.copy_(model.scan.scan_positions_m)
        for key, value in params.items():
            self.params[key].copy_(value)
        self.b.copy_(pieces["b"])
        self.layout.amplitude.copy_(pieces["layout"].amplitude)
        self.layout.coefficient_scale.copy_(pieces["layout"].coefficient_scale)
        self.normalization.copy_(pieces["normalization"])
        self.shift.copy_(pieces["shift"])

    def matvec(self, vector):
        grads, coefficient = self.model.vjp(self.params, self.b,
                                            self.model.jvp(self.params, self.b, *self.layout.unpack(vector)))  # fmt: skip
        return self.layout.pack_gradient(grads, coefficient) / self.normalization + self.shift * vector


_JOINT_GRAPHS = GraphCache()


def _graphed_joint_pcg(model, params, specs, config, pieces, rhs, diagonal):
    """The joint slide's conjugate gradients from a CUDA graph kept across slides (batched)."""
    from .linalg import GraphedPCG

    key = (tuple(model.shape), repr(model.scan.fmcw_config), model.fresnel_n, repr(specs), config.real,
           config.cg_iterations, config.cg_tolerance, rhs.shape, rhs.dtype, rhs.device,
           tuple((k, tuple(v.shape), v.dtype) for k, v in params.items()), pieces["b"].dtype)  # fmt: skip
    entry = _JOINT_GRAPHS.get(key)
    if entry is None:
        static = _StaticJoint(model, params, specs, pieces, not config.real)
        solver = GraphedPCG(static.matvec, rhs, diagonal, config.cg_iterations, config.cg_tolerance)
        _JOINT_GRAPHS[key] = entry = (static, solver)
    else:
        entry[0].refill(model, params, pieces)
    return entry[1].solve(rhs, diagonal)


@torch.no_grad()
def joint_slide(state, config, screen=None):
    """Joint Gauss-Newton steps, the system built on joint_apertures seeded apertures.

    The subset only shapes the proposal; acceptance refits on every observation.
    Returns the state and the number of accepted steps.
    """
    model, target = state.model, state.target
    if 0 < config.joint_apertures < model.apertures:
        ids, model = model.sample_apertures(config.joint_apertures, config.seed + state.iteration)
        target = target[ids]
    accepted = 0
    overlap = getattr(config, "batched", False) and screen is not None and target.is_cuda
    for inner in range(config.lm_steps):
        ready = None
        if overlap:  # the state's tensors are complete in stream order here
            ready = torch.cuda.Event()
            ready.record()
        pieces = {}
        with stage("slide.system"):
            matvec, gradient, diagonal, proposal = joint_system(
                model, state.params, state.coefficients, target, state.parameters, config,
                config.seed + state.iteration + inner, pieces=pieces)  # fmt: skip
        with stage("slide.pcg"):
            if getattr(config, "batched", False) and target.is_cuda and config.cg_iterations > 1 and \
                    hasattr(model, "scan"):  # fmt: skip
                delta = _graphed_joint_pcg(model, state.params, state.parameters, config, pieces, -gradient, diagonal)
            else:
                delta = pcg(matvec, -gradient, diagonal, iterations=config.cg_iterations,
                            tolerance=config.cg_tolerance, capture=getattr(config, "batched", False))  # fmt: skip
        if overlap:
            # The screening objective of the current geometry needs neither the system
            # nor its solution: it runs on a second stream while the conjugate gradients
            # (enqueued above) run on this one, and is simply unused if no step follows.
            current = torch.cuda.current_stream()
            side = side_stream(current.device)
            side.wait_event(ready)
            with torch.cuda.stream(side), stage("slide.screen"):
                bar = screen_bar(screen, state.params, config)
            current.wait_stream(side)
        descent = torch.isfinite(delta).all() & (delta @ gradient < 0)
        if not bool(descent):
            break
        if not overlap:
            with stage("slide.screen"):
                bar = screen_bar(screen, state.params, config)
        for fraction in BACKTRACK_JOINT:
            with stage("slide.accept"):
                trial = accept(state, proposal(delta, fraction), config, bar)
            if trial is not None:
                state, accepted = trial, accepted + 1
                break
        else:
            break
    return state, accepted
