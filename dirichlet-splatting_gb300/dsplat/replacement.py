"""Fixed-budget support replacement.

Both policies install a new support only when its refitted objective is lower.

utility  (one slot per step) swaps the least useful atom for the best certificate
         candidate;
merged   pools many candidates with the whole support, fits the pool once, ranks every
         pooled atom by what deleting it would cost, deletes the cheapest until the
         budget holds and lets surviving candidates take the freed slots.

Semantics of the reference's dsplat/replacement.py:27-270. The pooled fit is organized
around _PooledFit: the Gram of support + candidates is assembled from the state's own
support block and one cross product of all pooled rows against the new columns (a
tcgen05 launch in bf16x3 mode); the deletion order comes from backward elimination on its
regularized inverse (batched mode: one CUDA kernel per deletion on the inverse Cholesky
factor, which costs a quarter of forming the inverse).
"""

from __future__ import annotations

from dataclasses import replace

import torch

from .certificate import certificate
from .kernels import search
from .linalg import shifted_cholesky
from .normal import PROJECTIONS, TensorCoreGram, fused_rows, row_chunk
from .parameters import periodic_delta
from .tracing import stage
from .varpro import Fit, accept, refined_coefficients, rendered_loss, screen_bar, varpro


def _feasible(state, pool, owner):
    """The pool as feasible atoms; fields the pool lacks are copied from slot owner."""
    size = len(pool["centers"])
    atoms = {}
    for key, spec in state.parameters.items():
        donor = state.params[key][owner].expand(size, *state.params[key].shape[1:])
        atoms[key] = spec.project(pool.get(key, donor), donor)
    return atoms


# --- utility: one slot per step --------------------------------------------------------------


def _projection_efficiency(gram):
    """1 / sqrt(max(G^-1_jj G_jj, 1)) per atom; G+ on a singular Gram.

    A singular Gram marks a column redundant (efficiency 0) exactly when its coordinate
    takes part in the nullspace; zero columns are redundant too.
    """
    factor, status = torch.linalg.cholesky_ex(gram)
    scale = gram.diagonal().real
    if int(status) == 0:
        inverse_diag = torch.cholesky_inverse(factor).diagonal().real
        return (inverse_diag * scale).clamp(min=1).rsqrt()
    values, vectors = torch.linalg.eigh(gram)
    eps = torch.finfo(values.dtype).eps
    kept = values > values.abs().max() * len(values) * eps
    reciprocal = torch.where(kept, values.clamp(min=torch.finfo(values.dtype).tiny).reciprocal(), 0)
    weight = vectors.abs().square()
    inverse_diag = weight @ reciprocal
    in_null = (weight * (~kept)).sum(1) > len(values) * eps * 10
    efficiency = (inverse_diag * scale).clamp(min=1).rsqrt()
    return torch.where(in_null | (scale <= 0), 0, efficiency)


def utility(gram, coefficients):
    """Half relative amplitude, half unregularized projection efficiency, per atom."""
    magnitude = coefficients.abs()
    return 0.5 * magnitude / magnitude.max().clamp(min=1e-30) + 0.5 * _projection_efficiency(gram)


@torch.no_grad()
def replace_one(state, config, pool, screen=None):
    """Try the best pool candidate in the least useful slot; (state, atoms replaced)."""
    owner = int(utility(state.gram, state.coefficients).argmin())
    candidate = _feasible(state, pool, owner)
    scores = certificate(state.model, candidate, state.target - state.prediction, config.coefficients)
    if config.min_separation > 0:
        support, period = state.params["centers"], state.parameters["centers"].period
        for start in range(0, len(scores), 256):
            gap = periodic_delta(candidate["centers"][start : start + 256, None] - support[None], period)
            too_close = gap.norm(dim=-1).amin(1) < config.min_separation
            scores[start : start + 256].masked_fill_(too_close, -torch.inf)
    scores = torch.where(torch.isfinite(scores), scores, -torch.inf)
    best = scores.argmax()
    pick, positive = torch.stack((best.double(), (scores[best] > 0).double())).tolist()
    if not positive:
        return state, 0
    pick = int(pick)
    proposal = {key: value.clone() for key, value in state.params.items()}
    for key in proposal:
        proposal[key][owner] = candidate[key][pick]
    accepted = accept(state, proposal, config, screen_bar(screen, state.params, config))
    return (state, 0) if accepted is None else (accepted, 1)


# --- merged: pool candidates, fit once, prune back to the budget -----------------------------


def regularized_inverse(h, floor):
    """(h + floor lambda_max(h) I)^-1 in float64, or None."""
    with stage("inverse.cholesky"):
        factor = shifted_cholesky(h, floor)
    if factor is None:
        return None
    with stage("inverse.invert"):
        return torch.cholesky_inverse(factor)


def regularized_inverse_factor(h, floor):
    """X = L^-1 of the factor of regularized_inverse's shifted system (inverse = X^H X)."""
    with stage("inverse.cholesky"):
        factor = shifted_cholesky(h, floor)
    if factor is None:
        return None
    with stage("inverse.invert"):
        return search.triangular_inverse(factor)


def backward_elimination(inverse, rhs, count, limited=None, limit=0, *, on_device=False, factored=False):
    """Indices of count unknowns removed one at a time from a least-squares fit, in order.

    With W the inverse of the current normal matrix and b = W q, removing unknown j and
    refitting raises the objective by |b_j|^2 / W_jj. Each step removes the cheapest
    unknown, then updates b and the diagonal by the rank-one downdate
    W <- W - w w^H / W_jj (w = W[:, j]), kept as a list of scaled columns. At most limit
    of the unknowns flagged in limited may go. on_device runs one CUDA kernel per step
    (the same arithmetic up to the order of float64 sums); factored means inverse holds
    X with W = X^H X.
    """
    if factored:
        if on_device and inverse.is_cuda:
            return search.backward_elimination_factor(inverse, rhs, count, limited, limit)
        inverse = inverse.mH @ inverse
    if on_device and inverse.is_cuda:
        return search.backward_elimination(inverse, rhs, count, limited, limit)
    n = len(inverse)
    device = inverse.device
    b = inverse @ rhs.to(inverse.dtype)
    diag = inverse.diagonal().real.clone()
    tiny = torch.finfo(diag.dtype).tiny
    downdates = inverse.new_zeros((n, count))  # scaled columns w / sqrt(W_jj) of every removal
    gone = torch.zeros(n, dtype=torch.bool, device=device)
    order = torch.zeros(count, dtype=torch.long, device=device)
    used = torch.zeros((), dtype=torch.long, device=device)
    # every index below stays a device tensor (index_select / index_fill_): no value is read back
    for k in range(count):
        blocked = gone if limited is None else gone | (limited & (used >= limit))
        j = (b.abs().square() / diag.clamp(min=tiny)).masked_fill(blocked, torch.inf).argmin().reshape(1)
        w = inverse.index_select(1, j).squeeze(1)
        if k:
            w = w - downdates[:, :k] @ downdates.index_select(0, j).squeeze(0)[:k].conj()
        pivot = w.index_select(0, j).real.clamp(min=tiny)
        b = b - w * (b.index_select(0, j) / pivot)
        column = w / pivot.sqrt()
        downdates[:, k] = column
        diag = diag - column.abs().square()
        gone.index_fill_(0, j, True)
        diag.index_fill_(0, j, 1.0)  # keeps the masked cost of a removed unknown finite
        b.index_fill_(0, j, 0)
        order[k : k + 1] = j
        if limited is not None:
            used = used + limited.index_select(0, j).squeeze(0)
    return order


def _distinct(scores, points, occupied, period, separation, width):
    """Up to width best-scoring candidates colliding neither with occupied nor each other.

    A collision is a distance below separation, or exactly zero (one atom pooled twice
    would make the pooled system singular for nothing). Candidates are taken best first
    in blocks of 1024; inside a block a candidate yields only to a better kept one.
    """

    def distances(a, b):
        return periodic_delta(a[:, None] - b[None], period).norm(dim=-1)

    def clear(gap):
        return (gap >= separation) & (gap > 0)

    ranked = scores.argsort(descending=True, stable=True)
    ranked = ranked[torch.isfinite(scores[ranked])]
    kept, total = [], 0
    for start in range(0, len(ranked), 1024):
        if total >= width:
            break
        ids = ranked[start : start + 1024]
        block = points[ids]
        free = clear(distances(block, occupied).amin(1))
        for earlier in kept:
            free &= clear(distances(block, points[earlier]).amin(1))
        conflict = (~clear(distances(block, block))).triu(1)
        if bool(conflict[free][:, free].any()):
            for i in free.nonzero().flatten().tolist():
                if bool((conflict[:i, i] & free[:i]).any()):
                    free[i] = False
        kept.append(ids[free])
        total += int(free.sum())
    return torch.cat(kept)[:width] if kept else ranked[:0]


def _cross_on_tensor_cores(model, pool, target, support, chunk, support_params=None):
    """(cross [total, added] = A^T A[:, support:], right = A[:, support:]^T y), tcgen05 Gram.

    When the support's projected rows are still stored (normal.PROJECTIONS, found by the
    support's own parameter tensors) only the new atoms are projected, beside them.
    Returns the cross, the right-hand side and the cache entry now holding the pool's rows.
    """
    total = len(pool["centers"])
    entry = None if support_params is None else PROJECTIONS.find(model, support_params)
    if entry is not None and -(-total // 128) * 128 <= entry[2].n_alloc and entry[3] == chunk:
        store = entry[2]
        gram = TensorCoreGram(model, total, chunk, target.device, store=store)
        fresh = {key: value[support:] for key, value in pool.items()}
        status = fused_rows(model, fresh, store, chunk, first_unknown=support)
    else:
        gram = TensorCoreGram(model, total, chunk, target.device)
        status = fused_rows(model, pool, gram.store, chunk)
        entry = None
        if status is not None and support_params is not None:
            entry = PROJECTIONS.put(model, support_params, gram.store, chunk)
    if status is None:
        right = torch.zeros(total - support, dtype=torch.float64, device=target.device)
        for a, y in model.blocks(pool, target, True, chunk):
            gram.store.append(a)
            right += a[:, support:].T @ y
    else:
        from .kernels.gram import check

        right = model.correlate({key: value[support:] for key, value in pool.items()}, target)[0].real.double()
        check(status)
    products, _ = gram.finish(column_from=support)
    new = products[support:, support:]
    cross = torch.cat((products[:support, support:], torch.triu(new) + torch.triu(new, 1).T))
    return cross.float(), right.float(), entry


def pooled_statistics(state, pool, config, projections=None):
    """Gram and right-hand side of the support followed by the pooled new atoms.

    Only the new columns are streamed; the support block is the state's. projections, a
    list, receives the ProjectionCache entry holding the pool's rows (tensor-core path).
    """
    model, support = state.model, len(state.coefficients)
    total = len(pool["centers"])
    chunk = row_chunk(model, total, config)
    if config.real and getattr(config, "gram", "fp32") == "bf16x3":
        # The fused projection stores no dictionary block, so its block layout follows the
        # support's size, as the support's own refits do: the stored rows of a refit and
        # the pool's new rows then share one layout, and a pool gives the same Gram whether
        # or not the support's rows were still stored.
        fused_chunk = row_chunk(model, support, config)
        cross, right, entry = _cross_on_tensor_cores(model, pool, state.target, support, fused_chunk, state.params)
        if projections is not None:
            projections.append(entry)
    else:
        cross = state.gram.new_zeros((total, total - support))
        right = state.rhs.new_zeros(total - support)
        for a, y in model.blocks(pool, state.target, config.real, chunk):
            fresh = a[:, support:]
            cross.addmm_(a.mH, fresh)
            right.addmv_(fresh.mH, y)
    cross = cross / model.size
    gram = state.gram.new_empty((total, total))
    gram[:support, :support] = state.gram
    gram[:, support:] = cross
    gram[support:, :] = cross.mH
    gram[support:, support:] = (cross[support:] + cross[support:].mH) * 0.5
    rhs = torch.cat((state.rhs, right / model.size))
    return gram, rhs


def _all_free(spec):
    flags = spec.trainable
    return all(bool(f) for f in flags) if isinstance(flags, (tuple, list)) else bool(flags)


class _PooledFit:
    """One regularized fit of support + candidates and the deletions it ranks."""

    def __init__(self, state, pool, config):
        self.state, self.pool, self.config = state, pool, config
        self.support = len(state.coefficients)
        self.projections = []
        with stage("replace.pooled"):
            self.gram, self.rhs = pooled_statistics(state, pool, config, self.projections)
        h = self.gram.real if config.real else self.gram
        if config.ridge:
            h = h.clone()
            h.diagonal().add_(config.ridge)
        self.q = self.rhs.real if config.real else self.rhs
        self.batched = getattr(config, "batched", False)
        self.factored = self.batched and h.is_cuda
        floor = len(h) * torch.finfo(h.real.dtype).eps
        with stage("replace.inverse"):
            self.inverse = (regularized_inverse_factor if self.factored else regularized_inverse)(h, floor)
        self.is_old = torch.arange(len(self.q), device=self.q.device) < self.support

    def survivors(self, deletions, limit):
        """(slot -> pooled index map, owners: old slots that left) after the deletions."""
        with stage("replace.elimination"):
            removed = backward_elimination(self.inverse, self.q, deletions, None if limit is None else self.is_old,
                                           limit or 0, on_device=self.batched, factored=self.factored)  # fmt: skip
        dropped = torch.zeros(len(self.q), dtype=torch.bool, device=self.q.device)
        dropped[removed] = True
        owners = dropped[: self.support].nonzero().flatten()
        slots = torch.arange(self.support, device=self.q.device)
        if len(owners):
            slots[owners] = (~dropped[self.support :]).nonzero().flatten() + self.support
        return slots, owners

    def trial(self, slots, owners):
        """Support of the surviving atoms (new atoms take their slot's frozen fields) and its fit."""
        state = self.state
        atoms = {key: value[slots] for key, value in self.pool.items()}
        # new atoms copied slot 0's frozen fields when pooled; they take the ones of the
        # slot they fill, and then their pooled columns no longer apply
        moved = False
        for key, spec in state.parameters.items():
            if _all_free(spec):
                continue
            fixed = spec.project(atoms[key][owners], state.params[key][owners])
            moved = moved or not torch.equal(fixed, atoms[key][owners])
            atoms[key][owners] = fixed
        if moved:
            with stage("replace.refit"):
                return atoms, varpro(state.model, atoms, state.target, self.config)
        gram = self.gram[slots[:, None], slots[None, :]]
        rhs = self.rhs[slots]
        coefficients = refined_coefficients(state.model, atoms, state.target, gram, rhs, self.config)
        prediction, objective = rendered_loss(state.model, atoms, coefficients, state.target, self.config.ridge)
        return atoms, Fit(coefficients, prediction, objective, gram, rhs)


@torch.no_grad()
def merge_support(state, config, pool, scores=None):
    """Pool the best candidates with the support, fit once, prune back to the budget.

    The pooled fit ranks old and new atoms by the cost of deleting them; the cheapest
    leave until the budget is met, and surviving new atoms take the slots of old atoms
    that left. The result must lower the rendered objective; a rejected support is
    retried allowing half as many old atoms to leave. Returns (state, atoms replaced).
    """
    support = state.params["centers"]
    candidate = _feasible(state, pool, 0)
    if scores is None:
        scores = certificate(state.model, candidate, state.target - state.prediction, config.coefficients)
    with stage("replace.distinct"):
        period = state.parameters["centers"].period
        pick = search.distinct if getattr(config, "batched", False) else _distinct
        chosen = pick(scores, candidate["centers"], support, period, config.min_separation, config.batch)
    if not len(chosen):
        return state, 0
    pooled = {key: torch.cat((value, candidate[key][chosen])) for key, value in state.params.items()}
    fit = _PooledFit(state, pooled, config)
    if fit.inverse is None:
        return state, 0
    limit = None
    while True:
        slots, owners = fit.survivors(len(chosen), limit)
        if not len(owners):
            return state, 0
        atoms, result = fit.trial(slots, owners)
        if result.objective < state.objective:
            entry = fit.projections[0] if fit.projections else None
            if entry is not None and PROJECTIONS.find(state.model, state.params) is entry:
                PROJECTIONS.adopt(entry, slots, owners, atoms)  # the next pool starts from it
            return replace(state, params=atoms, **result._asdict()), len(owners)
        limit = len(owners) // 2
        if limit < 1:
            return state, 0
