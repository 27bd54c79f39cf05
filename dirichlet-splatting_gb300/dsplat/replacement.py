"""Fixed-budget support replacement.

Both policies install a new support only if its refitted objective is lower.
utility swaps the least useful atom for the best certificate candidate; merged pools
many candidates with the whole support, ranks every atom by the cost of deleting it
from one pooled fit and keeps the budget's cheapest-to-lose complement. Behaviour
follows the reference's dsplat/replacement.py:27-270.
"""

from __future__ import annotations

from dataclasses import replace

import torch

from .certificate import certificate
from .kernels import search
from .parameters import periodic_delta
from .tracing import stage
from .varpro import (
    Fit,
    accept,
    fit_coefficients,
    rendered_loss,
    row_chunk,
    screen_bar,
    shifted_cholesky,
    varpro,
)


def _feasible(state, pool, owner):
    """The pool as feasible atoms; fields the pool lacks copy slot owner."""
    count = len(pool["centers"])
    result = {}
    for key, spec in state.parameters.items():
        reference = state.params[key][owner].expand(count, *state.params[key].shape[1:])
        result[key] = spec.project(pool.get(key, reference), reference)
    return result


# --- utility: one slot per step --------------------------------------------------------------


def utility(gram, coefficients):
    """Half relative amplitude, half unregularized projection efficiency of every atom.

    Efficiency is 1 / sqrt(G^-1_jj G_jj). For a singular Gram a column is redundant
    exactly when its coordinate takes part in the nullspace; the others use G+.
    """
    chol, info = torch.linalg.cholesky_ex(gram)
    diag = gram.diag().real
    if int(info) == 0:
        inverse_diag = torch.cholesky_inverse(chol).diag().real
        efficiency = (1 / (inverse_diag * diag).clamp(min=1)).sqrt()
    else:
        values, vectors = torch.linalg.eigh(gram)
        eps = torch.finfo(values.dtype).eps
        active = values > values.abs().max() * len(values) * eps
        inv = torch.where(active, values.clamp(min=torch.finfo(values.dtype).tiny).reciprocal(), 0)
        inverse_diag = (vectors.abs().square() * inv[None]).sum(1)
        null_weight = vectors[:, ~active].abs().square().sum(1)
        efficiency = (1 / (inverse_diag * diag).clamp(min=1)).sqrt()
        efficiency = torch.where(null_weight > len(values) * eps * 10, 0, efficiency)
        efficiency = torch.where(diag > 0, efficiency, 0)
    magnitude = coefficients.abs()
    return 0.5 * magnitude / magnitude.max().clamp(min=1e-30) + 0.5 * efficiency


@torch.no_grad()
def replace_one(state, config, pool, screen=None):
    """Try the best pool candidate in the least useful slot; the state and atoms replaced."""
    owner = int(utility(state.gram, state.coefficients).argmin())
    candidate = _feasible(state, pool, owner)
    residual = state.target - state.prediction
    scores = certificate(state.model, candidate, residual, config.coefficients)
    if config.min_separation > 0:
        centers, period = state.params["centers"], state.parameters["centers"].period
        for start in range(0, len(scores), 256):
            delta = periodic_delta(candidate["centers"][start : start + 256, None] - centers[None], period)
            near = delta.norm(dim=-1).min(1).values < config.min_separation
            scores[start : start + 256][near] = -torch.inf
    scores[~torch.isfinite(scores)] = -torch.inf
    index = int(scores.argmax())
    if not scores[index] > 0:
        return state, 0
    proposal = {key: value.clone() for key, value in state.params.items()}
    for key in proposal:
        proposal[key][owner] = candidate[key][index]
    accepted = accept(state, proposal, config, screen_bar(screen, state.params, config))
    return (state, 0) if accepted is None else (accepted, 1)


# --- merged: pool candidates, fit once, prune back to the budget -----------------------------


def regularized_inverse(h, floor):
    """Inverse of h + floor lambda_max(h) I in double precision, or None."""
    with stage("inverse.cholesky"):
        factor = shifted_cholesky(h, floor)
    if factor is None:
        return None
    with stage("inverse.invert"):
        return torch.cholesky_inverse(factor)


def regularized_inverse_factor(h, floor):
    """X = L^-1 with L the factor of regularized_inverse's shifted system (inverse = X^H X).

    The batched replacement eliminates from X: a triangular inverse (trtri) costs a quarter
    of forming the inverse (potri) at float64 on this GPU.
    """
    with stage("inverse.cholesky"):
        factor = shifted_cholesky(h, floor)
    if factor is None:
        return None
    with stage("inverse.invert"):
        return search.triangular_inverse(factor)


def backward_elimination(inverse, rhs, count, limited=None, limit=0, *, on_device=False, factored=False):
    """Remove count unknowns one at a time from the least squares with this inverse.

    With W the inverse of the current system and b = W q, deleting unknown j and
    refitting raises the objective by |b_j|^2 / W_jj; each step deletes the cheapest
    and continues with W - w w^H / W_jj (w = W[:, j]), kept as rank-one corrections.
    At most limit of the unknowns marked in limited are removed. Returns the removed
    indices in order. on_device runs the loop as one CUDA kernel per step
    (dsg_backward_elimination) instead of about ten PyTorch launches; the arithmetic is
    the same up to the order of the float64 sums. factored means inverse is the factor X
    of regularized_inverse_factor (the inverse being X^H X).
    """
    if factored:
        if on_device and inverse.is_cuda:
            return search.backward_elimination_factor(inverse, rhs, count, limited, limit)
        inverse = inverse.mH @ inverse
    if on_device and inverse.is_cuda:
        return search.backward_elimination(inverse, rhs, count, limited, limit)
    size = len(inverse)
    b = inverse @ rhs.to(inverse.dtype)
    diagonal = inverse.diagonal().real.clone()
    alive = torch.ones(size, device=inverse.device, dtype=torch.bool)
    updates = inverse.new_zeros((size, count))
    removed = torch.zeros(count, device=inverse.device, dtype=torch.long)
    spent = torch.zeros((), device=inverse.device, dtype=torch.long)
    tiny = torch.finfo(diagonal.dtype).tiny
    # Indexing with device tensors (index_select / index_fill_) keeps every step on the
    # device: no value is read back, so the loop can also be captured in a CUDA graph.
    for step in range(count):
        cost = b.abs().square() / diagonal.clamp(min=tiny)
        blocked = ~alive if limited is None else ~alive | (limited & (spent >= limit))
        index = cost.masked_fill(blocked, torch.inf).argmin().view(1)
        column = inverse.index_select(1, index)[:, 0]
        if step:
            column = column - updates[:, :step] @ updates.index_select(0, index)[0, :step].conj()
        pivot = column.index_select(0, index).real.clamp(min=tiny)
        b = b - column * (b.index_select(0, index) / pivot)
        scaled = column / pivot.sqrt()
        updates[:, step] = scaled
        diagonal = diagonal - scaled.abs().square()
        alive.index_fill_(0, index, False)
        diagonal.index_fill_(0, index, 1.0)  # a removed unknown stays masked; this keeps its cost finite
        b.index_fill_(0, index, 0)
        removed[step : step + 1] = index
        if limited is not None:
            spent = spent + limited.index_select(0, index)[0]
    return removed


def _distinct(scores, points, occupied, period, separation, width):
    """Best-scoring candidates colliding neither with the support nor with each other.

    A collision is a distance below separation, or exactly zero (an atom pooled twice
    would make the pooled system singular for no gain).
    """

    def distance(a, b):
        return periodic_delta(a[:, None] - b[None], period).norm(dim=-1)

    order = scores.argsort(descending=True, stable=True)
    order = order[torch.isfinite(scores[order])]
    kept, found = [], 0
    for start in range(0, len(order), 1024):
        if found >= width:
            break
        ids = order[start : start + 1024]
        block = points[ids]
        near = distance(block, occupied).min(1).values
        free = (near >= separation) & (near > 0)
        for previous in kept:
            near = distance(block, points[previous]).min(1).values
            free &= (near >= separation) & (near > 0)
        inside = distance(block, block)
        clash = ((inside < separation) | (inside == 0)).triu(1)
        if bool(clash[free][:, free].any()):
            # Greedy by score: a candidate yields only to a kept better one.
            for i in free.nonzero().flatten().tolist():
                if bool((clash[:i, i] & free[:i]).any()):
                    free[i] = False
        kept.append(ids[free])
        found += int(free.sum())
    return torch.cat(kept)[:width] if kept else order[:0]


def pooled_statistics(state, pool, config):
    """Gram and right-hand side over the support followed by the pooled new atoms.

    Only the new columns are streamed; the support block is the state's. With
    DSFWConfig.gram == "bf16x3" (real coefficients) the cross products of all pooled
    rows against the new columns are one tcgen05 launch over the stored split rows.
    """
    model, count = state.model, len(state.coefficients)
    total, added = len(pool["centers"]), len(pool["centers"]) - count
    gram = state.gram.new_empty((total, total))
    rhs = state.rhs.new_empty(total)
    gram[:count, :count], rhs[:count] = state.gram, state.rhs
    chunk = row_chunk(model, total, config)
    if config.real and getattr(config, "gram", "fp32") == "bf16x3":
        cross, right = _pooled_cross_mixed(model, pool, state.target, count, added, chunk, config)
    else:
        cross = state.gram.new_zeros((total, added))
        right = state.rhs.new_zeros(added)
        for a, y in model.blocks(pool, state.target, config.real, chunk):
            new = a[:, count:]
            cross.addmm_(a.H, new)
            right.addmv_(new.H, y)
    cross /= model.size
    gram[:, count:], gram[count:, :] = cross, cross.H
    gram[count:, count:] = (cross[count:] + cross[count:].H) * 0.5
    rhs[count:] = right / model.size
    return gram, rhs


def _pooled_cross_mixed(model, pool, target, count, added, chunk, config):
    """cross [total, added] = A^T A[:, count:] and right = A[:, count:]^T y on the tensor cores."""
    from .kernels.gram import GramRows, check
    from .varpro import fused_rows, projected_rows

    total = count + added
    device = target.device
    store = GramRows(total, projected_rows(model, chunk), device)
    fused = fused_rows(model, pool, store, chunk)
    if fused is not None:
        new = {key: value[count:] for key, value in pool.items()}
        right = model.correlate(new, target)[0].real.double()
        check(fused)
    else:
        right = torch.zeros(added, dtype=torch.float64, device=device)
        for a, y in model.blocks(pool, target, True, chunk):
            store.append(a)
            right += a[:, count:].T @ y
    products = torch.zeros((total, total), dtype=torch.float64, device=device)
    check(store.accumulate(products, column_from=count))
    cross = torch.empty((total, added), dtype=torch.float64, device=device)
    cross[:count] = products[:count, count:]
    block = products[count:, count:]
    cross[count:] = torch.triu(block) + torch.triu(block, 1).T
    return cross.to(torch.float32), right.to(torch.float32)


@torch.no_grad()
def merge_support(state, config, pool, scores=None):
    """Pool the best candidates with the support, fit once, prune back to the budget.

    One regularized pooled fit ranks old and new atoms by the cost of deleting them;
    the cheapest leave until the budget is met and surviving new atoms take the slots
    of old atoms that left. The result needs a lower rendered objective; a rejected
    support is retried with half as many old atoms allowed to leave. Returns the state
    and the number of atoms replaced.
    """
    centers = state.params["centers"]
    count = len(centers)
    candidate = _feasible(state, pool, 0)
    if scores is None:
        residual = state.target - state.prediction
        scores = certificate(state.model, candidate, residual, config.coefficients)
    with stage("replace.distinct"):
        period = state.parameters["centers"].period
        if getattr(config, "batched", False):
            chosen = search.distinct(scores, candidate["centers"], centers, period,
                                     config.min_separation, config.batch)  # fmt: skip
        else:
            chosen = _distinct(scores, candidate["centers"], centers, period, config.min_separation,
                               config.batch)  # fmt: skip
    if not len(chosen):
        return state, 0
    pool = {key: torch.cat((value, candidate[key][chosen])) for key, value in state.params.items()}
    with stage("replace.pooled"):
        gram, rhs = pooled_statistics(state, pool, config)
    real = config.real
    eye = torch.eye(len(gram), dtype=gram.dtype, device=gram.device)
    h = (gram.real if real else gram) + config.ridge * eye
    factored = getattr(config, "batched", False) and h.is_cuda
    with stage("replace.inverse"):
        floor = len(h) * torch.finfo(h.real.dtype).eps
        inverse = regularized_inverse_factor(h, floor) if factored else regularized_inverse(h, floor)
    if inverse is None:
        return state, 0
    q = rhs.real if real else rhs
    old = torch.arange(len(q), device=q.device) < count
    limit = None
    while True:
        with stage("replace.elimination"):
            removed = backward_elimination(inverse, q, len(chosen), None if limit is None else old,
                                           limit or 0, on_device=getattr(config, "batched", False),
                                           factored=factored)  # fmt: skip
        gone = torch.zeros(len(q), device=q.device, dtype=torch.bool)
        gone[removed] = True
        owners = gone[:count].nonzero().flatten()
        if not len(owners):
            return state, 0
        ids = torch.arange(count, device=q.device)
        ids[owners] = (~gone[count:]).nonzero().flatten() + count
        trial = {key: value[ids] for key, value in pool.items()}
        # New atoms copied slot 0's frozen components; they take those of the slot they
        # fill, and then their pooled columns no longer apply.
        moved = False
        for key, spec in state.parameters.items():
            if not spec.mask(trial[key]).all():
                fixed = spec.project(trial[key][owners], state.params[key][owners])
                moved = moved or not torch.equal(fixed, trial[key][owners])
                trial[key][owners] = fixed
        if moved:
            with stage("replace.refit"):
                fit = varpro(state.model, trial, state.target, config)
        else:
            trial_gram, trial_rhs = gram[ids[:, None], ids[None, :]], rhs[ids]
            b = fit_coefficients(trial_gram, trial_rhs, config)
            fit = Fit(b, *rendered_loss(state.model, trial, b, state.target, config.ridge),
                      trial_gram, trial_rhs)  # fmt: skip
        if fit.objective < state.objective:
            return replace(state, params=trial, **fit._asdict()), len(owners)
        limit = len(owners) // 2
        if limit < 1:
            return state, 0
