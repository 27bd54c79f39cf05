"""Variable projection: streamed normal equations, coefficient elimination and acceptance.

Objective: mean(|A b - y|^2) + ridge |b|^2. Complex coefficients use the full Gram
G = A^H A / M; signed-real coefficients use Re(G) and Re(q). A new geometry is kept
only if its refitted objective is lower. Behaviour follows the reference's
dsplat/varpro.py:17-228; the Gram products run on libdsplat_gb300.so (plain FP32
SYRK) or, with DSFWConfig.gram == "bf16x3", on the tcgen05 split-BF16x3 kernel.
"""

from __future__ import annotations

from dataclasses import replace
from typing import NamedTuple

import torch

from .kernels.cublas import syrk
from .kernels.reduce import energy
from .tracing import stage


class Fit(NamedTuple):
    """VarPro solution of one geometry; the field names match DSFWState."""

    coefficients: torch.Tensor
    prediction: torch.Tensor
    objective: float
    gram: torch.Tensor  # Re(A^H A) / M for real coefficients, A^H A / M otherwise
    rhs: torch.Tensor


POWER_STEPS = 24  # power iterations for the largest eigenvalue of a Gram
SHIFT_RETRIES = 4
FOLD = 8  # float32 blocks summed before each float64 fold of the Gram


def largest_eigenvalue(h):
    """Power-iteration estimate of the largest eigenvalue of a positive semidefinite h.

    The start vector is a fixed golden-ratio sequence, so the estimate is reproducible.
    """
    start = (torch.arange(len(h), device=h.device, dtype=torch.float64) * 0.6180339887) % 1 + 0.5
    vector = start.to(h.dtype)
    top = vector.norm()
    for _ in range(POWER_STEPS):
        vector = h @ vector
        top = vector.norm()
        vector = vector / top.clamp(min=torch.finfo(top.dtype).tiny)
    return top


def shifted_cholesky(h, floor):
    """Cholesky factor of h + shift I in double precision, or None.

    The shift starts at floor times lambda_max(h) and, while factorization fails,
    grows by 9x the accumulated shift (1, 10, 91, ... times), at most SHIFT_RETRIES times.
    """
    matrix = h.to(torch.complex128 if h.is_complex() else torch.float64, copy=True)
    shift = floor * largest_eigenvalue(matrix)
    for _ in range(SHIFT_RETRIES):
        matrix.diagonal().add_(shift)
        factor, info = torch.linalg.cholesky_ex(matrix)
        if int(info) == 0:
            return factor
        shift = shift * 9
    return None


def refined_solve(h, rhs, iterations=3, tolerance=1e-13):
    """Solve of a float64 system from a float32 Cholesky factor with float64 refinement.

    On this GPU a float32 factorization costs a seventh of the float64 one; each
    refinement step is a float64 residual and a float32 triangular solve pair. Returns
    None (the caller then factors in float64) when the float32 factor fails or the
    normwise backward error |q - h x| / (|h|_F |x| + |q|) stays above tolerance, which
    happens only for systems whose condition number approaches 1 / float32 epsilon. One
    device read decides both.
    """
    low = torch.complex64 if h.is_complex() else torch.float32
    chol, info = torch.linalg.cholesky_ex(h.to(low))
    q = rhs[:, None] if rhs.ndim == 1 else rhs
    q = q.to(h.dtype)
    x = torch.cholesky_solve(q.to(low), chol).to(h.dtype)
    for _ in range(iterations):
        x = x + torch.cholesky_solve((q - h @ x).to(low), chol).to(h.dtype)
    error = (q - h @ x).norm() / (torch.linalg.matrix_norm(h) * x.norm() + q.norm()).clamp(min=1e-300)
    if not bool((info == 0) & (error <= tolerance)):  # a failed factor leaves NaN in error
        return None
    return x[:, 0] if rhs.ndim == 1 else x


def solve(h, rhs, refined=False):
    """Hermitian solve; a singular system is shifted to where a pseudoinverse would truncate.

    The shift len(h) eps lambda_max only moves the solution along near-null directions,
    which the prediction does not see. refined solves the shifted float64 system with
    refined_solve (float32 factor, float64 refinement) before factoring it in float64;
    both give its solution to float64 accuracy before the cast back to the input type.
    """
    q = rhs[:, None] if rhs.ndim == 1 else rhs
    chol, info = torch.linalg.cholesky_ex(h)
    if int(info) != 0:
        floor = len(h) * torch.finfo(h.real.dtype).eps
        if refined and h.is_cuda:
            x = shifted_refined_solve(h, q, floor)
            if x is not None:
                return (x[:, 0] if rhs.ndim == 1 else x).to(rhs.dtype)
        chol = shifted_cholesky(h, floor)
    if chol is None:  # every column is zero: nothing to fit
        return torch.zeros_like(rhs)
    x = torch.cholesky_solve(q.to(chol.dtype), chol).to(q.dtype)
    return x[:, 0] if rhs.ndim == 1 else x


def shifted_refined_solve(h, q, floor):
    """(h + floor lambda_max(h) I)^-1 q at the first shift of shifted_cholesky, or None."""
    matrix = h.to(torch.complex128 if h.is_complex() else torch.float64, copy=True)
    matrix.diagonal().add_(floor * largest_eigenvalue(matrix))
    return refined_solve(matrix, q)


def row_chunk(model, columns, config):
    """Observation rows per streamed block: bounded elements, whole apertures."""
    chunk = min(config.row_chunk, max(1, config.dictionary_elements // columns))
    return max(model.row_alignment, chunk - chunk % model.row_alignment)


def _gram_mode(config):
    return getattr(config, "gram", "fp32")


def projected_rows(model, chunk):
    """Number of real rows model.blocks(..., real=True, chunk) yields, known before streaming."""
    if hasattr(model, "block_basis"):
        bins = model.shape[1]
        total = 0
        for start in range(0, model.size, chunk):
            rows = slice(start, min(start + chunk, model.size))
            basis = model.block_basis(rows)
            width = 2 * bins if basis is None else basis.interleaved.shape[0]
            total += width * (-(-rows.stop // bins) - rows.start // bins)
        return total
    return 2 * model.size


def fused_rows(model, params, store, chunk):
    """Store every projected real row block with the fused design-projection kernel.

    Returns the kernel status tensor, or None (nothing stored) when the model or any
    block's basis is outside what the fused kernel covers; the caller then streams.
    """
    from .kernels.gram import append_projected, fused_supported

    if not hasattr(model, "block_basis"):
        return None
    config, positions = model.sensor
    bins = model.shape[1]
    runs = []  # consecutive blocks sharing one basis: (first aperture, last aperture, basis)
    for start in range(0, model.size, chunk):
        rows = slice(start, min(start + chunk, model.size))
        basis = model.block_basis(rows)
        if not fused_supported(config, basis):
            return None
        first, last = rows.start // bins, rows.stop // bins
        if runs and runs[-1][2] is basis and runs[-1][1] == first:
            runs[-1] = (runs[-1][0], last, basis)
        else:
            runs.append((first, last, basis))
    status = torch.zeros(1, dtype=torch.int32, device=positions.device)
    for first, last, basis in runs:
        append_projected(store, config, positions[first:last], params, basis, model.fresnel_n, status)
    return status


def normal_equations(model, params, target, config):
    """G = A^H A / M and q = A^H y / M, streamed over projected row blocks.

    Real blocks accumulate the upper triangle in float32 (SYRK) and fold it into a
    float64 total every FOLD blocks. In the bf16x3 mode every block is stored split
    and transposed, and one tcgen05 launch adds the whole Gram to the float64 total.
    """
    count = len(params["centers"])
    chunk = row_chunk(model, count, config)
    stream = model.blocks(params, target, config.real, chunk)
    if not config.real:
        gram = target.new_zeros((count, count))
        rhs = target.new_zeros(count)
        for a, y in stream:
            gram.addmm_(a.H, a)
            rhs.addmv_(a.H, y)
        return (gram + gram.H) / (2 * model.size), rhs / model.size
    device = target.device
    total = torch.zeros((count, count), dtype=torch.float64, device=device)
    rhs = torch.zeros(count, dtype=torch.float64, device=device)
    if _gram_mode(config) == "bf16x3":
        from .kernels.gram import GramRows, check

        store = GramRows(count, projected_rows(model, chunk), device)
        fused = fused_rows(model, params, store, chunk)
        if fused is not None:
            rhs += model.correlate(params, target)[0].real.double()
            check(fused)
        else:
            for a, y in stream:
                store.append(a)
                rhs += a.T @ y
        check(store.accumulate(total))
    else:
        part = torch.zeros((count, count), dtype=torch.float32, device=device)
        for index, (a, y) in enumerate(stream):
            a = a.contiguous()
            syrk(a, part)
            rhs += a.T @ y
            if index % FOLD == FOLD - 1:
                total += part
                part.zero_()
        total += part
    gram = (torch.triu(total) + torch.triu(total, 1).T) / model.size
    return gram.float(), (rhs / model.size).float()


def fit_coefficients(gram, rhs, config):
    """Minimizer of b^H G b - 2 Re(b^H q) + ridge |b|^2 in the configured domain.

    With DSFWConfig.batched a system that needs solve's shifted float64 factorization is
    first solved by refined_solve; the coefficients agree to float64 accuracy either way.
    """
    if config.real:
        gram, rhs = gram.real, rhs.real
    eye = torch.eye(len(gram), dtype=gram.dtype, device=gram.device)
    return solve(gram + config.ridge * eye, rhs, refined=getattr(config, "batched", False))


def rendered_loss(model, params, coefficients, target, ridge):
    """Prediction and the complete objective; the data term is summed in float64."""
    prediction = model.render(params, coefficients)
    penalty = coefficients.abs().square().sum().double()
    loss = energy(prediction, target) / model.size + ridge * penalty
    return prediction, float(loss)


@torch.no_grad()
def varpro(model, params, target, config):
    """Coefficients, prediction, objective, Gram and right-hand side of one geometry."""
    with stage("varpro.normal"):
        gram, rhs = normal_equations(model, params, target, config)
    with stage("varpro.solve"):
        b = fit_coefficients(gram, rhs, config)
    with stage("varpro.loss"):
        return Fit(b, *rendered_loss(model, params, b, target, config.ridge), gram, rhs)


@torch.no_grad()
def exchange_varpro(state, proposal, slot, config):
    """VarPro after one atom changed: only its Gram column and right-hand side are new."""
    model, target = state.model, state.target
    atom = {key: value[slot : slot + 1] for key, value in proposal.items()}
    column = model.render(atom, target.real.new_ones(1))
    cross = model.correlate(proposal, column)[0] / model.size
    value = (column.conj() * target).sum() / model.size
    if config.real:
        cross, value = cross.real, value.real
    gram, rhs = state.gram.clone(), state.rhs.clone()
    gram[:, slot] = cross
    gram[slot, :] = cross.conj()
    gram[slot, slot] = cross[slot].real
    rhs[slot] = value
    b = fit_coefficients(gram, rhs, config)
    return Fit(b, *rendered_loss(model, proposal, b, target, config.ridge), gram, rhs)


def screen_bar(screen, params, config):
    """(model, target, subset objective of params) of an aperture subset, or None."""
    if screen is None:
        return None
    model, target = screen
    return model, target, varpro(model, params, target, config).objective


@torch.no_grad()
def accept(state, proposal, config, screen=None):
    """The state with proposal installed if its refitted objective is lower, else None.

    One changed atom refits only its Gram column. A screen from screen_bar first
    rejects proposals that are clearly worse on its aperture subset.
    """
    changed = torch.zeros(len(state.coefficients), dtype=torch.bool, device=state.target.device)
    for key, value in proposal.items():
        changed |= (value != state.params[key]).reshape(len(changed), -1).any(-1)
    slots = changed.nonzero().flatten().tolist()
    if not slots:
        return None
    if screen is not None:
        model, target, bar = screen
        if varpro(model, proposal, target, config).objective > bar + 1e-4 * state.power:
            return None
    if len(slots) == 1:
        fit = exchange_varpro(state, proposal, slots[0], config)
    else:
        fit = varpro(state.model, proposal, state.target, config)
    if not fit.objective < state.objective:
        return None
    return replace(state, params=proposal, **fit._asdict())


def pcg(operator, rhs, diagonal, *, iterations=32, tolerance=1e-3):
    """Jacobi-preconditioned conjugate gradients from zero."""
    x = torch.zeros_like(rhs)
    norm = rhs.norm()
    r = rhs.clone()
    z = r / diagonal
    p = z.clone()
    rz = r @ z
    for _ in range(iterations):
        hp = operator(p)
        curvature = p @ hp
        if not curvature > 0:
            break
        alpha = rz / curvature
        x += alpha * p
        r -= alpha * hp
        if r.norm() <= tolerance * norm:
            break
        z = r / diagonal
        next_rz = r @ z
        p = z + (next_rz / rz) * p
        rz = next_rz
    return x
