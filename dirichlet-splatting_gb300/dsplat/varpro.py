"""Variable projection: coefficient elimination, objective and acceptance of a geometry.

Objective: mean(|A b - y|^2) + ridge |b|^2. For a fixed geometry the coefficients are a
linear least-squares solution, so the solver only ever compares geometries by their
refitted objective ("VarPro"): complex coefficients use G = A^H A / M, signed-real ones
Re(G) and Re(q). A proposal is kept only when its refitted objective is lower. Semantics
of the reference's dsplat/varpro.py:17-203. The normal equations are dsplat.normal
(FP32 SSYRK or the tcgen05 split-BF16x3 Gram), the solves dsplat.linalg, the objective's
data term the fixed-order float64 dsg_energy reduction.
"""

from __future__ import annotations

from dataclasses import replace
from typing import NamedTuple

import torch

from .kernels.reduce import energy
from .linalg import (  # noqa: F401  (names of the reference's varpro module)
    POWER_STEPS,
    SHIFT_RETRIES,
    factored_solver,
    largest_eigenvalue,
    pcg,
    refined_solve,
    shifted_cholesky,
    shifted_refined_solve,
    solve,
)
from .normal import FOLD, fused_rows, normal_equations, projected_rows, row_chunk  # noqa: F401
from .graphs import side_stream
from .tracing import stage


class Fit(NamedTuple):
    """VarPro solution of one geometry; the field names match DSFWState."""

    coefficients: torch.Tensor
    prediction: torch.Tensor
    objective: float
    gram: torch.Tensor  # Re(A^H A) / M for real coefficients, A^H A / M otherwise
    rhs: torch.Tensor


def fit_coefficients(gram, rhs, config):
    """argmin_b b^H G b - 2 Re(b^H q) + ridge |b|^2 in the configured coefficient domain.

    Batched mode (DSFWConfig.batched) solves a system that needs the shifted float64
    factor from a float32 factor with float64 refinement; both agree to float64 accuracy.
    """
    h, q = (gram.real, rhs.real) if config.real else (gram, rhs)
    if config.ridge:
        h = h.clone()
        h.diagonal().add_(config.ridge)
    return solve(h, q, refined=getattr(config, "batched", False))


RESIDUAL_REFINEMENTS = 1  # coefficient refinements against the rendered residual (bf16x3 Gram)


def _refines(config):
    """Whether coefficients from this configuration's Gram are refined against the residual."""
    return config.real and getattr(config, "gram", "fp32") == "bf16x3"


def refined_coefficients(model, params, target, gram, rhs, config):
    """Coefficients of the normal equations, refined against the true residual.

    The split-BF16x3 Gram carries relative errors near 3e-5 of its largest entry, which the
    solve amplifies by the Gram's condition number. Each refinement renders the current
    fit with the exact forward kernel, correlates the float32 residual with every atom
    (dsg_surfel_correlate: g = Re(A^H (y - A b)) / M - ridge b, the residual of the normal
    equations with the exact operator) and adds the correction solved with the same Gram:
    iterative refinement with the approximate Gram as the preconditioner, converging to
    the coefficients of the exact least-squares problem.
    """
    if not _refines(config):
        return fit_coefficients(gram, rhs, config)
    h, q = gram.real, rhs.real
    if config.ridge:
        h = h.clone()
        h.diagonal().add_(config.ridge)
    solve_with = factored_solver(h, refined=getattr(config, "batched", False))
    b = solve_with(q)
    for _ in range(RESIDUAL_REFINEMENTS):
        residual = target - model.render(params, b)
        g = model.correlate(params, residual)[0].real / model.size
        if config.ridge:
            g = g - config.ridge * b
        b = b + solve_with(g.to(q.dtype)).to(b.dtype)
    return b


def rendered_loss(model, params, coefficients, target, ridge):
    """(prediction, objective) of coefficients; the data term is summed in float64."""
    prediction = model.render(params, coefficients)
    data = energy(prediction, target) / model.size
    penalty = coefficients.abs().square().sum().double()
    return prediction, float(data + ridge * penalty)


def _refit(model, params, target, config, gram, rhs):
    coefficients = refined_coefficients(model, params, target, gram, rhs, config)
    prediction, objective = rendered_loss(model, params, coefficients, target, config.ridge)
    return Fit(coefficients, prediction, objective, gram, rhs)


@torch.no_grad()
def varpro(model, params, target, config, normal=None):
    """Coefficients, prediction, objective, Gram and right-hand side of one geometry.

    normal, when given, is this geometry's (Gram, right-hand side), already formed.
    """
    if normal is not None:
        gram, rhs = normal
    else:
        with stage("varpro.normal"):
            gram, rhs = normal_equations(model, params, target, config)
    with stage("varpro.solve"):
        coefficients = refined_coefficients(model, params, target, gram, rhs, config)
    with stage("varpro.loss"):
        prediction, objective = rendered_loss(model, params, coefficients, target, config.ridge)
    return Fit(coefficients, prediction, objective, gram, rhs)


@torch.no_grad()
def exchange_varpro(state, proposal, slot, config):
    """VarPro after one atom changed: only its Gram row / column and right-hand side change.

    The new column is the atom rendered alone with a unit coefficient, correlated with
    every atom of the proposal (one correlation launch) and with the data.
    """
    model, target = state.model, state.target
    single = {key: value[slot : slot + 1] for key, value in proposal.items()}
    column = model.render(single, target.real.new_ones(1))
    cross = model.correlate(proposal, column)[0] / model.size
    value = (column.conj() * target).sum() / model.size
    if config.real:
        cross, value = cross.real, value.real
    gram = state.gram.clone()
    gram[:, slot] = cross
    gram[slot, :] = cross.conj()
    gram[slot, slot] = cross[slot].real
    rhs = state.rhs.clone()
    rhs[slot] = value
    return _refit(model, proposal, target, config, gram, rhs)


def screen_bar(screen, params, config):
    """(model, target, subset objective of params) of an aperture subset, or None."""
    if screen is None:
        return None
    model, target = screen
    return model, target, varpro(model, params, target, config).objective


def changed_slots(params, proposal):
    """(number of atoms whose fields differ, index of the first one), in one device read."""
    first_field = next(iter(params.values()))
    count = len(first_field)
    differs = torch.zeros(count, dtype=torch.bool, device=first_field.device)
    for key, value in proposal.items():
        differs |= (value != params[key]).reshape(count, -1).any(-1)
    total, first = torch.stack((differs.sum(), differs.to(torch.int8).argmax())).tolist()
    return total, first


def _early_normal(state, proposal, config):
    """The full normal equations of proposal, enqueued on a second stream (batched mode).

    The screening refit that decides whether they are needed is latency bound (small
    kernels and a few device reads), so the large projection and Gram launches of the full
    system run beside it instead of after it; a rejected proposal only wastes them.
    """
    current = torch.cuda.current_stream()
    side = side_stream(current.device)
    side.wait_stream(current)
    with torch.cuda.stream(side), stage("varpro.normal"):
        normal, statuses = normal_equations(state.model, proposal, state.target, config, deferred=True)
    return side, normal, statuses


def _finish_normal(early):
    """(Gram, right-hand side) of _early_normal, ordered after its stream and checked."""
    from .kernels.gram import check

    side, normal, statuses = early
    current = torch.cuda.current_stream()
    current.wait_stream(side)
    for tensor in (*normal, *statuses):
        tensor.record_stream(current)  # made on the side stream, used and freed on this one
    for status in statuses:
        check(status)
    return normal


@torch.no_grad()
def accept(state, proposal, config, screen=None):
    """The state with proposal installed if its refitted objective is lower, else None.

    A screen from screen_bar first rejects proposals that are clearly worse on its
    aperture subset (by more than 1e-4 of the data power); one changed atom refits only
    its Gram column, more refit the whole geometry.
    """
    total, first = changed_slots(state.params, proposal)
    if total == 0:
        return None
    early = None
    if screen is not None:
        model, target, bar = screen
        if total > 1 and getattr(config, "batched", False) and state.target.is_cuda:
            early = _early_normal(state, proposal, config)
        if varpro(model, proposal, target, config).objective > bar + 1e-4 * state.power:
            if early is not None:
                torch.cuda.current_stream().wait_stream(early[0])  # its memory is reused after this
            return None
    if total == 1:
        fit = exchange_varpro(state, proposal, first, config)
    elif early is not None:
        fit = varpro(state.model, proposal, state.target, config, normal=_finish_normal(early))
    else:
        fit = varpro(state.model, proposal, state.target, config)
    if not fit.objective < state.objective:
        return None
    return replace(state, params=proposal, **fit._asdict())
