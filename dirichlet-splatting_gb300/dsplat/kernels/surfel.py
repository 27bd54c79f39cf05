"""FMCW surfel kernels behind the reference's binding signatures.

Replaces dsplat/kernels/surfel.py of the reference (slangtorch launches of
surfel.slang and correlate.slang) with calls into libdsplat_gb300.so. config is an
FMCWConfig, positions the sensor positions [A, 3]; weights are per-surfel complex
amplitudes (reflectivity times sqrt(area)); the area chain lives in dsplat.surfel.
Complex gradients follow PyTorch: dL/dx = Re(conj(upstream) dy/dx).
"""

from __future__ import annotations

from contextlib import contextmanager

import torch
from torch.autograd.function import once_differentiable

from . import _lib
from ._lib import call, f32, ptr, real_view


# FP32 flops per counting unit (pair-bin; pair-normal for the normal bank) used for the
# roofline accounting of the FP32-issue-bound kernels.
FLOPS_PER_UNIT = {
    "dsg_surfel_render": 16, "dsg_surfel_render_samples": 6, "dsg_surfel_jvp": 24, "dsg_surfel_vjp": 20, "dsg_surfel_correlate": 18,
    "dsg_surfel_correlate_active": 18, "dsg_surfel_correlate_gradient": 30,
    "dsg_surfel_correlate_orientations": 12, "dsg_surfel_orient_best": 12,
}  # fmt: skip


# DSG_TUNE_CORRELATION_FORM: how correlate, correlate_active, correlate_gradient and vjp
# evaluate their sums over range bins.
CORRELATION_FORMS = {"auto": 0, "exact": 1, "interp": 2}
_CORRELATION_FORM_KNOB = 3


@contextmanager
def correlation_form(name):
    """Inside the block the aperture-reduced kernels use form name: "interp" (the default:
    per-pair statistics interpolated from per-aperture tables, a type-2 nonuniform FFT)
    or "exact" (the closed-form kernel summed over every bin)."""
    previous = int(_lib.library().dsg_tuning_get(_CORRELATION_FORM_KNOB))
    call("dsg_tuning_set", _CORRELATION_FORM_KNOB, CORRELATION_FORMS[name])
    try:
        yield
    finally:
        call("dsg_tuning_set", _CORRELATION_FORM_KNOB, previous)


def _work(name, units):
    _lib.add_work(name, float(units) * FLOPS_PER_UNIT[name])


def _tuned(family, config, apertures, surfels, device):
    """Set the library's launch-shape knob of family for this shape (dsplat.autotune)."""
    from .. import autotune

    autotune.apply(family, apertures=apertures, surfels=surfels, bins=config.num_range_bins, pad=config.pad_factor,
                   device=device)  # fmt: skip


def _outputs(centers, *shape, dtype=torch.float32):
    return torch.empty(shape, dtype=dtype, device=centers.device)


# How the forward evaluates the profiles: "bins" sums the closed-form kernel over the range
# bins (dsg_surfel_render); "samples" sums the pairs' ADC samples by phasor recurrence and
# takes the N-point FFT (dsg_surfel_render_samples + cuFFT).
RENDER_FORMS = ("bins", "samples")
_RENDER_FORM = ["bins"]


@contextmanager
def render_form(name):
    """Inside the block the forward uses form name ("bins", the default, or "samples")."""
    if name not in RENDER_FORMS:
        raise KeyError(name)
    previous, _RENDER_FORM[0] = _RENDER_FORM[0], name
    try:
        yield
    finally:
        _RENDER_FORM[0] = previous


def render_samples(config, positions, centers, normals, weights, fresnel_n, status=None):
    """ADC samples y [A, S] complex64 whose N-point FFT's first K bins are the profiles.

    status, an int32 device tensor of one element, is set to 1 if a surfel copy never
    arrived (the affected samples are then NaN); by default a scratch word is used.
    """
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    w = real_view(weights)
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    out = _outputs(centers, apertures, config.adc_samples, 2)
    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device=centers.device)
    nbytes = _lib.query("dsg_surfel_render_samples_workspace_bytes", chirp, apertures, count)
    work, nbytes = _lib.workspace(nbytes, centers.device)
    _work("dsg_surfel_render_samples", len(positions) * len(centers) * config.adc_samples)
    call(
        "dsg_surfel_render_samples", chirp, ptr(positions), apertures, ptr(centers), ptr(normals), ptr(w),
        count, ptr(out), ptr(work), nbytes, ptr(status), _lib.stream(centers.device),
    )  # fmt: skip
    return torch.view_as_complex(out)


def _profiles(config, positions, centers, normals, weights, fresnel_n):
    """Range profiles [A, K, 2] of weights [S, 2] (interleaved complex)."""
    if _RENDER_FORM[0] == "samples":
        samples = render_samples(config, positions, centers, normals, torch.view_as_complex(weights.contiguous()),
                                 fresnel_n)  # fmt: skip
        spectrum = torch.fft.fft(samples, n=config.n_fft, dim=1)[:, : config.num_range_bins]
        return torch.view_as_real(spectrum.contiguous()).contiguous()
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    weights = weights.contiguous()
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    out = _outputs(centers, apertures, config.num_range_bins, 2)
    nbytes = _lib.query("dsg_surfel_render_workspace_bytes", chirp, apertures, count)
    work, nbytes = _lib.workspace(nbytes, centers.device)
    _work("dsg_surfel_render", len(positions) * len(centers) * config.num_range_bins)
    call(
        "dsg_surfel_render", chirp, ptr(positions), apertures, ptr(centers), ptr(normals),
        ptr(weights), count, ptr(out), ptr(work), nbytes, _lib.stream(centers.device),
    )  # fmt: skip
    return out


def vjp(config, positions, centers, normals, weights, upstream, fresnel_n):
    """Gradients of Re(conj(upstream) . profiles) for centers, normals and complex weights."""
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    w, u = real_view(weights), real_view(upstream)
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    gc, gn, gw = (_outputs(centers, count, 3), _outputs(centers, count, 3),
                  _outputs(centers, count, 2))  # fmt: skip
    nbytes = _lib.query("dsg_surfel_reduce_workspace_bytes", chirp, apertures, count, 8)
    work, nbytes = _lib.workspace(nbytes, centers.device)
    _work("dsg_surfel_vjp", apertures * count * config.num_range_bins)
    call(
        "dsg_surfel_vjp", chirp, ptr(positions), apertures, ptr(centers), ptr(normals), ptr(w),
        count, ptr(u), ptr(gc), ptr(gn), ptr(gw), ptr(work), nbytes,
        _lib.stream(centers.device),
    )  # fmt: skip
    return gc, gn, torch.view_as_complex(gw)


def jvp(config, positions, centers, normals, weights, delta_centers, delta_normals,
        delta_weights, fresnel_n):  # fmt: skip
    """Directional derivative of the profiles [A, K]."""
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    dc, dn = f32(delta_centers), f32(delta_normals)
    w, dw = real_view(weights), real_view(delta_weights)
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    out = _outputs(centers, apertures, config.num_range_bins, 2)
    nbytes = _lib.query("dsg_surfel_render_workspace_bytes", chirp, apertures, count)
    work, nbytes = _lib.workspace(nbytes, centers.device)
    _work("dsg_surfel_jvp", apertures * count * config.num_range_bins)
    call(
        "dsg_surfel_jvp", chirp, ptr(positions), apertures, ptr(centers), ptr(normals), ptr(w),
        ptr(dc), ptr(dn), ptr(dw), count, ptr(out), ptr(work), nbytes,
        _lib.stream(centers.device),
    )  # fmt: skip
    return torch.view_as_complex(out)


def render_scenes(scenes):
    """Profiles of many scenes in one persistent launch (dsg_surfel_render_scenes).

    scenes: sequence of (config, positions [A, 3], centers [S, 3], normals [S, 3], weights
    [S] complex, fresnel_n) on one device; every config needs pad 2 and 128 or 256 range
    bins. Returns the profiles [A, K] complex64 of each scene, in order.
    """
    if not scenes:
        return []
    device = scenes[0][1].device
    keep, outputs = [], []  # every buffer the kernel reads stays referenced until the launch is queued
    table = (_lib.RenderScene * len(scenes))()
    for slot, (config, positions, centers, normals, weights, fresnel_n) in zip(table, scenes, strict=True):
        pos, cen, nrm, w = f32(positions), f32(centers), f32(normals), real_view(weights)
        out = torch.empty((len(pos), config.num_range_bins, 2), dtype=torch.float32, device=device)
        keep += [pos, cen, nrm, w]
        outputs.append(out)
        slot.chirp = _lib.chirp(config, fresnel_n)
        slot.positions, slot.apertures = pos.data_ptr() if len(pos) else None, len(pos)
        slot.centers = cen.data_ptr() if len(cen) else None
        slot.normals = nrm.data_ptr() if len(nrm) else None
        slot.weights = w.data_ptr() if len(w) else None
        slot.surfels, slot.out = len(cen), out.data_ptr() if len(pos) else None
        _work("dsg_surfel_render", len(pos) * len(cen) * config.num_range_bins)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    nbytes = _lib.query("dsg_surfel_render_scenes_workspace_bytes", table, len(scenes))
    work, nbytes = _lib.workspace(nbytes, device)
    call("dsg_surfel_render_scenes", table, len(scenes), ptr(work), nbytes, ptr(status), _lib.stream(device))
    if int(status.item()) != 0:
        raise _lib.DsplatKernelError("dsg_surfel_render_scenes: a scene descriptor was rejected on the device")
    del keep
    return [torch.view_as_complex(out) for out in outputs]


class _Render(torch.autograd.Function):
    """Profiles forward; the backward is the hand-written adjoint kernel (dsg_surfel_vjp)."""

    @staticmethod
    def forward(ctx, centers, normals, weights, positions, config, fresnel_n):
        ctx.save_for_backward(centers, normals, weights, positions)
        ctx.config, ctx.fresnel_n = config, fresnel_n
        return _profiles(config, positions, centers, normals, weights, fresnel_n)

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        centers, normals, weights, positions = ctx.saved_tensors
        upstream = torch.view_as_complex(grad.contiguous())
        gc, gn, gw = vjp(
            ctx.config, positions, centers, normals, torch.view_as_complex(weights), upstream,
            ctx.fresnel_n,
        )  # fmt: skip
        return gc, gn, torch.view_as_real(gw), None, None, None


def render(config, positions, centers, normals, weights, fresnel_n):
    """Range profiles [A, K]; differentiable in centers, normals and weights."""
    output = _Render.apply(
        centers.contiguous(), normals.contiguous(), real_view(weights), positions, config, fresnel_n
    )
    return torch.view_as_complex(output)


def design(config, positions, centers, normals, areas, fresnel_n, real):
    """Dictionary rows of whole apertures including sqrt(area).

    Complex rows are [A * K, S]; real rows are [2 * A * K, S] ordered bin by bin,
    row (2 k + part) * A + a, so one product projects every aperture onto a row basis.
    """
    positions, centers, normals, areas = f32(positions), f32(centers), f32(normals), f32(areas)
    chirp = _lib.chirp(config, fresnel_n)
    count, rows = len(centers), len(positions) * config.num_range_bins
    out = _outputs(centers, 2 * rows, count) if real else _outputs(centers, rows, count, 2)
    call(
        "dsg_surfel_design", chirp, ptr(positions), len(positions), ptr(centers), ptr(normals),
        ptr(areas), count, int(bool(real)), ptr(out), _lib.stream(centers.device),
    )  # fmt: skip
    return out if real else torch.view_as_complex(out)


def jacobian(config, positions, centers, normals, fresnel_n):
    """Columns [A, K, S] and their center and normal derivatives [A, K, S, 3], without area."""
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    chirp = _lib.chirp(config, fresnel_n)
    shape = (len(positions), config.num_range_bins, len(centers))
    cols = _outputs(centers, *shape, 2)
    jac = _outputs(centers, *shape, 6, 2)
    call(
        "dsg_surfel_jacobian", chirp, ptr(positions), len(positions), ptr(centers), ptr(normals),
        len(centers), ptr(cols), ptr(jac), _lib.stream(centers.device),
    )  # fmt: skip
    jac = torch.view_as_complex(jac)
    return torch.view_as_complex(cols), jac[..., :3], jac[..., 3:]


def interpolated():
    """Whether the aperture-reduced kernels run in the interpolated form (the default)."""
    return int(_lib.library().dsg_tuning_get(_CORRELATION_FORM_KNOB)) != CORRELATION_FORMS["exact"]


def residual_tables(config, residual, derivative=True, out=None):
    """Aperture tables of a residual [A, K] for the interpolated correlations (float32, flat).

    Computed once, they serve every correlate / correlate_gradient call given them
    (tables=...) with the same residual: the per-residual product of the interpolated form
    then runs once instead of once per call. derivative=False makes the correlation tables
    only (enough for correlate). out, when given, is filled in place (a static buffer).
    """
    r = real_view(residual)
    chirp = _lib.chirp(config)
    apertures = r.shape[0]
    nbytes = _lib.query("dsg_surfel_residual_tables_bytes", chirp, apertures, int(bool(derivative)))
    if out is None:
        out = torch.empty(nbytes // 4, dtype=torch.float32, device=r.device)
    elif out.numel() * 4 < nbytes:
        raise _lib.DsplatKernelError("residual tables buffer too small")
    call("dsg_surfel_residual_tables", chirp, ptr(r), apertures, int(bool(derivative)), ptr(out), out.numel() * 4,
         _lib.stream(r.device))  # fmt: skip
    return out


def correlate(config, positions, centers, normals, residual, fresnel_n, active=None, tables=None):
    """conj(column) . residual and |column|^2 per candidate, without area.

    active = (count, period), count an int32 device tensor of one element: only candidates
    whose index mod period is below count are computed; the others get zeros. tables, from
    residual_tables(residual), replaces residual (the same results, bitwise).
    """
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    corr, norm = _outputs(centers, count, 2), _outputs(centers, count)
    name = "dsg_surfel_correlate" if active is None else "dsg_surfel_correlate_active"
    _work(name, apertures * count * config.num_range_bins)
    if tables is not None:
        nbytes = _lib.query("dsg_surfel_tabled_workspace_bytes", apertures, count, 3)
        work, nbytes = _lib.workspace(nbytes, centers.device)
        limit, period = (None, 1) if active is None else (ptr(active[0]), int(active[1]))
        call(
            "dsg_surfel_correlate_tabled", chirp, ptr(positions), apertures, ptr(centers), ptr(normals), count,
            ptr(tables), limit, period, ptr(corr), ptr(norm), ptr(work), nbytes, _lib.stream(centers.device),
        )  # fmt: skip
        return torch.view_as_complex(corr), norm
    r = real_view(residual)
    nbytes = _lib.query("dsg_surfel_reduce_workspace_bytes", chirp, apertures, count, 3)
    work, nbytes = _lib.workspace(nbytes, centers.device)
    if active is None:
        call(
            "dsg_surfel_correlate", chirp, ptr(positions), apertures, ptr(centers), ptr(normals),
            count, ptr(r), ptr(corr), ptr(norm), ptr(work), nbytes, _lib.stream(centers.device),
        )  # fmt: skip
    else:
        limit, period = active
        call(
            "dsg_surfel_correlate_active", chirp, ptr(positions), apertures, ptr(centers),
            ptr(normals), count, ptr(r), ptr(limit), int(period), ptr(corr), ptr(norm), ptr(work),
            nbytes, _lib.stream(centers.device),
        )  # fmt: skip
    return torch.view_as_complex(corr), norm


def correlate_orientations(config, positions, centers, normals, bank, residual, fresnel_n,
                           table=None):  # fmt: skip
    """Correlations and norms [S, 1 + bank] for the current normal and every bank normal.

    table, an fmcw.RangeTable, replaces the per-bin sum by FFT-interpolated range
    correlations; it only ranks proposals. Without area.
    """
    positions, centers, normals, bank = f32(positions), f32(centers), f32(normals), f32(bank)
    chirp = _lib.chirp(config, fresnel_n)
    count = len(centers)
    _tuned("orient", config, len(positions), 0, centers.device)
    out = _outputs(centers, count, len(bank) + 1, 3)
    if table is None:
        r, rt, nt, oversample = real_view(residual), None, None, 1
    else:
        r, rt, nt = None, f32(table.correlation), f32(table.norm)
        oversample = table.oversample
    _work("dsg_surfel_correlate_orientations", len(positions) * count * (len(bank) + 1))
    call(
        "dsg_surfel_correlate_orientations", chirp, ptr(positions), len(positions), ptr(centers),
        ptr(normals), count, ptr(bank) if len(bank) else None, len(bank), ptr(r), ptr(rt),
        ptr(nt), oversample, ptr(out), _lib.stream(centers.device),
    )  # fmt: skip
    return torch.complex(out[..., 0], out[..., 1]), out[..., 2]


def orient_best(config, positions, centers, normals, areas, bank, residual, fresnel_n, energy, real_mode,
                table=None):  # fmt: skip
    """(which [S] int64, top [S] float32): each candidate's best normal (0 = its own, j = bank
    row j - 1) and its certificate, as correlate_orientations scaled by the areas and the
    selection of certificate.orient_candidates, in one launch. energy: a float64 device
    scalar (the residual's energy)."""
    positions, centers, normals, bank, areas = f32(positions), f32(centers), f32(normals), f32(bank), f32(areas)
    chirp = _lib.chirp(config, fresnel_n)
    count = len(centers)
    _tuned("orient", config, len(positions), 0, centers.device)
    which = _outputs(centers, count, dtype=torch.int32)
    top = _outputs(centers, count)
    if table is None:
        r, rt, nt, oversample = real_view(residual), None, None, 1
    else:
        r, rt, nt = None, f32(table.correlation), f32(table.norm)
        oversample = table.oversample
    energy = energy.to(torch.float64).reshape(1).contiguous()
    _work("dsg_surfel_orient_best", len(positions) * count * (len(bank) + 1))
    call(
        "dsg_surfel_orient_best", chirp, ptr(positions), len(positions), ptr(centers), ptr(normals), ptr(areas),
        count, ptr(bank) if len(bank) else None, len(bank), ptr(r), ptr(rt), ptr(nt), oversample, ptr(energy),
        int(bool(real_mode)), ptr(which), ptr(top), _lib.stream(centers.device),
    )  # fmt: skip
    return which.long(), top


def correlate_gradient(config, positions, centers, normals, residual, fresnel_n, include_normals, tables=None):
    """Correlation, norm and their center (and normal) derivatives [S, 3 or 6], without area.

    tables, from residual_tables(residual) with derivative, replaces residual (the same
    results, bitwise)."""
    positions, centers, normals = f32(positions), f32(centers), f32(normals)
    width = 6 if include_normals else 3
    chirp = _lib.chirp(config, fresnel_n)
    count, apertures = len(centers), len(positions)
    _tuned("splat", config, apertures, count, centers.device)
    corr, norm = _outputs(centers, count, 2), _outputs(centers, count)
    dcorr, dnorm = _outputs(centers, count, width, 2), _outputs(centers, count, width)
    _work("dsg_surfel_correlate_gradient", apertures * count * config.num_range_bins)
    if tables is not None:
        nbytes = _lib.query("dsg_surfel_tabled_workspace_bytes", apertures, count, 3 + 3 * width)
        work, nbytes = _lib.workspace(nbytes, centers.device)
        call(
            "dsg_surfel_correlate_gradient_tabled", chirp, ptr(positions), apertures, ptr(centers), ptr(normals),
            count, ptr(tables), width, ptr(corr), ptr(norm), ptr(dcorr), ptr(dnorm), ptr(work), nbytes,
            _lib.stream(centers.device),
        )  # fmt: skip
    else:
        r = real_view(residual)
        nbytes = _lib.query("dsg_surfel_reduce_workspace_bytes", chirp, apertures, count, 3 + 3 * width)
        work, nbytes = _lib.workspace(nbytes, centers.device)
        call(
            "dsg_surfel_correlate_gradient", chirp, ptr(positions), apertures, ptr(centers),
            ptr(normals), count, ptr(r), width, ptr(corr), ptr(norm), ptr(dcorr), ptr(dnorm),
            ptr(work), nbytes, _lib.stream(centers.device),
        )  # fmt: skip
    return (
        torch.view_as_complex(corr),
        norm,
        torch.view_as_complex(dcorr),
        dnorm,
    )
