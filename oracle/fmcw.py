"""Float64 FMCW surfel oracle on the CPU (test infrastructure; never product code).

Closed form of one dictionary column (reference: dsplat/groundtruth.py:40-55 _echoes,
tests/reference/oracle.py:34-41 fmcw_columns, dsplat/kernels/scattering.slang:16-50):

    r = |p - c|, u = (p - c) / r, cos = u . n
    col[a, k, s] = cos^2 F(cos) lambda / (8 pi r) exp(2 pi i (fc tau + K tau (t0 - tau/2)))
                   * D(k - r / spacing),    tau = 2 r / c0,  zero when cos <= 0

Derivatives come from PyTorch autograd of this float64 closed form, so they are
independent of the hand-derived adjoint of the CUDA kernels. Every function works on
aperture chunks to bound memory; config is any object with the FMCWConfig fields.
"""

from __future__ import annotations

import math

import torch

from .kernel import dirichlet

DTYPE = torch.float64


def _d(x):
    return torch.as_tensor(x).to(DTYPE)


def echoes(positions, centers, normals, config, fresnel_n=0.0):
    """Range [A, S] and complex echo amplitude [A, S] of each aperture-surfel pair."""
    diff = _d(positions)[:, None, :] - _d(centers)[None, :, :]
    distance = diff.norm(dim=-1).clamp(min=1e-9)
    cosine = (diff / distance[..., None] * _d(normals)[None]).sum(-1).clamp(min=0)
    amplitude = cosine.square() * config.lambda_m / (8 * math.pi * distance)
    if fresnel_n > 1:
        root = torch.sqrt(fresnel_n * fresnel_n - 1 + cosine.square())
        amplitude = amplitude * (root - cosine) / (root + cosine)
    tau = 2 * distance / config.c0_m_s
    cycles = config.fc_hz * tau + config.slope_hz_s * tau * (config.adc_start_time_s - 0.5 * tau)
    return distance, amplitude * torch.exp(2j * math.pi * cycles)


def columns(positions, centers, normals, config, fresnel_n=0.0):
    """Range-profile columns [A, K, S] in complex128, without area."""
    distance, amplitude = echoes(positions, centers, normals, config, fresnel_n)
    bins = torch.arange(config.num_range_bins, dtype=DTYPE)
    delta = bins[None, :, None] - distance[:, None, :] / config.range_bin_spacing_m
    return dirichlet(delta, config.adc_samples, config.n_fft)[0] * amplitude[:, None, :]


def _chunks(count, size):
    for start in range(0, count, size):
        yield slice(start, min(count, start + size))


def _complex(value):
    value = torch.as_tensor(value)
    return value.to(torch.complex128) if value.is_complex() else value.to(DTYPE).to(torch.complex128)


def render(config, positions, centers, normals, weights, fresnel_n=0.0, chunk=64):
    """Profiles [A, K] = columns @ weights in complex128."""
    w = _complex(weights)
    parts = [columns(positions[rows], centers, normals, config, fresnel_n) @ w
             for rows in _chunks(len(positions), chunk)]  # fmt: skip
    return torch.cat(parts)


@torch.enable_grad()
def vjp(config, positions, centers, normals, weights, upstream, fresnel_n=0.0, chunk=64):
    """Gradients of Re(conj(upstream) . render) for centers, normals and complex weights.

    Float64 autograd of the closed form; the weight gradient follows PyTorch's complex
    convention (sum of conj(column) * upstream).
    """
    c = _d(centers).clone().requires_grad_()
    n = _d(normals).clone().requires_grad_()
    w = _complex(weights).clone().requires_grad_()
    u = _complex(upstream)
    gc, gn, gw = torch.zeros_like(c), torch.zeros_like(n), torch.zeros_like(w)
    for rows in _chunks(len(positions), chunk):
        value = (u[rows].conj() * (columns(positions[rows], c, n, config, fresnel_n) @ w)).real.sum()
        a, b, d = torch.autograd.grad(value, (c, n, w))
        gc += a
        gn += b
        gw += d
    return gc.detach(), gn.detach(), gw.detach()


def jvp(config, positions, centers, normals, weights, delta_centers, delta_normals, delta_weights,
        fresnel_n=0.0, chunk=64):  # fmt: skip
    """Directional derivative [A, K] of render along (delta_centers, delta_normals, delta_weights).

    Forward-mode AD of the float64 closed form (torch.func.jvp).
    """
    c, n, w = _d(centers), _d(normals), _complex(weights)
    dc, dn, dw = _d(delta_centers), _d(delta_normals), _complex(delta_weights)
    parts = []
    for rows in _chunks(len(positions), chunk):
        block = positions[rows]

        def function(cc, nn, ww):
            return columns(block, cc, nn, config, fresnel_n) @ ww

        parts.append(torch.func.jvp(function, (c, n, w), (dc, dn, dw))[1])
    return torch.cat(parts)


def design(config, positions, centers, normals, areas, fresnel_n=0.0, real=False):
    """Dictionary rows including sqrt(area): complex [A K, S], or real [2 A K, S] bin-major."""
    cols = columns(positions, centers, normals, config, fresnel_n) * _d(areas).sqrt()
    A, K, S = cols.shape
    if not real:
        return cols.reshape(A * K, S)
    parts = torch.view_as_real(cols)  # [A, K, S, 2]
    return parts.permute(1, 3, 0, 2).reshape(2 * K * A, S)  # row (2k + part) * A + a


def correlate(config, positions, centers, normals, residual, fresnel_n=0.0, chunk=64):
    """conj(column) . residual and |column|^2 per candidate, without area."""
    r = _complex(residual)
    corr = torch.zeros(len(centers), dtype=torch.complex128)
    norm = torch.zeros(len(centers), dtype=DTYPE)
    for rows in _chunks(len(positions), chunk):
        cols = columns(positions[rows], centers, normals, config, fresnel_n)
        corr += (cols.conj() * r[rows][:, :, None]).sum((0, 1))
        norm += cols.abs().square().sum((0, 1))
    return corr, norm


@torch.enable_grad()
def correlate_gradient(config, positions, centers, normals, residual, fresnel_n=0.0,
                       include_normals=False, chunk=64):  # fmt: skip
    """corr, norm and their derivatives by centers (and normals), [C, 3 or 6], float64 autograd."""
    c = _d(centers).clone().requires_grad_()
    n = _d(normals).clone().requires_grad_()
    r = _complex(residual)
    width = 6 if include_normals else 3
    corr = torch.zeros(len(centers), dtype=torch.complex128)
    norm = torch.zeros(len(centers), dtype=DTYPE)
    d_re = torch.zeros((len(centers), width), dtype=DTYPE)
    d_im = torch.zeros_like(d_re)
    d_norm = torch.zeros_like(d_re)
    for rows in _chunks(len(positions), chunk):
        cols = columns(positions[rows], c, n, config, fresnel_n)
        value = (cols.conj() * r[rows][:, :, None]).sum((0, 1))
        energy = cols.abs().square().sum((0, 1))
        for target, out in ((value.real.sum(), d_re), (value.imag.sum(), d_im), (energy.sum(), d_norm)):
            gc, gn = torch.autograd.grad(target, (c, n), retain_graph=True)
            out[:, :3] += gc
            if include_normals:
                out[:, 3:] += gn
        corr += value.detach()
        norm += energy.detach()
    return corr, norm, torch.complex(d_re, d_im), d_norm


def correlate_orientations(config, positions, centers, normals, bank, residual, fresnel_n=0.0,
                           table=None, chunk=64):  # fmt: skip
    """Correlations and norms [C, 1 + bank] for each candidate's own normal and every bank normal.

    Without table the per-aperture correlation is the exact bin sum; with a
    (correlation [A, n_fft*ov, 2], norm [n_fft*ov], oversample) table it is the
    Catmull-Rom interpolation at r / spacing * oversample (dsplat/kernels/correlate.slang:133-146).
    """
    cen, own, bank = _d(centers), _d(normals), _d(bank)
    pos = _d(positions)
    count = len(cen)
    corr = torch.zeros((count, 1 + len(bank)), dtype=torch.complex128)
    norm = torch.zeros((count, 1 + len(bank)), dtype=DTYPE)
    for rows in _chunks(len(pos), chunk):
        p = pos[rows]
        diff = p[:, None, :] - cen[None]
        distance = diff.norm(dim=-1).clamp(min=1e-9)
        u = diff / distance[..., None]
        tau = 2 * distance / config.c0_m_s
        cycles = config.fc_hz * tau + config.slope_hz_s * tau * (config.adc_start_time_s - 0.5 * tau)
        rot = torch.exp(2j * math.pi * cycles)
        if table is None:
            bins = torch.arange(config.num_range_bins, dtype=DTYPE)
            delta = bins[None, :, None] - distance[:, None, :] / config.range_bin_spacing_m
            kern = dirichlet(delta, config.adc_samples, config.n_fft)[0]  # [a, K, C]
            r = _complex(residual)[rows]
            per = (kern.conj() * r[:, :, None]).sum(1) * rot.conj()  # [a, C]
            pnorm = kern.abs().square().sum(1)
        else:
            correlation, ntable, oversample = table
            correlation = torch.view_as_complex(_d(correlation).contiguous())[rows]
            ntable = _d(ntable)
            size = ntable.numel()
            x = distance / config.range_bin_spacing_m * oversample
            base = torch.floor(x)
            t = x - base
            weights = [-0.5 * t + t**2 - 0.5 * t**3, 1 - 2.5 * t**2 + 1.5 * t**3,
                       0.5 * t + 2 * t**2 - 1.5 * t**3, -0.5 * t**2 + 0.5 * t**3]  # fmt: skip
            value = torch.zeros_like(rot)
            pnorm = torch.zeros_like(distance)
            for j in range(4):
                k = (base.long() + j - 1) % size
                value = value + weights[j] * torch.gather(correlation, 1, k)
                pnorm = pnorm + weights[j] * ntable[k]
            per = value * rot.conj()
            pnorm = pnorm.clamp(min=0)
        normals_all = torch.cat((own[None].expand(len(p), -1, -1)[..., None, :],
                                 bank[None, None].expand(len(p), count, -1, -1)), 2)  # [a, C, 1+B, 3]
        cosine = (u[:, :, None, :] * normals_all).sum(-1)
        amp = torch.where(cosine > 0, cosine.square() * config.lambda_m / (8 * math.pi * distance[..., None]), 0)
        if fresnel_n > 1:
            cc = cosine.clamp(min=0)
            root = torch.sqrt(fresnel_n * fresnel_n - 1 + cc.square())
            amp = amp * (root - cc) / (root + cc)
        corr += (amp * per[..., None]).sum(0)
        norm += (amp.square() * pnorm[..., None]).sum(0)
    return corr, norm


def synthesize(positions, centers, normals, amplitudes, config, fresnel_n=0.0):
    """ADC-domain scan [A, K] (complex128): beat tones summed in float64, then range FFT / S.

    Independent of the Dirichlet kernel (dsplat/groundtruth.py:58-90).
    """
    time = torch.arange(config.adc_samples, dtype=DTYPE) / config.sample_rate_hz
    amps = _complex(amplitudes)
    profiles = []
    for rows in _chunks(len(positions), 128):
        adc = torch.zeros((rows.stop - rows.start, config.adc_samples), dtype=torch.complex128)
        for part in _chunks(len(centers), 512):
            distance, echo = echoes(positions[rows], centers[part], normals[part], config, fresnel_n)
            beat = 2 * config.slope_hz_s * distance / config.c0_m_s
            adc += ((echo * amps[part])[:, :, None] * torch.exp(2j * math.pi * beat[:, :, None] * time)).sum(1)
        profiles.append(torch.fft.fft(adc, n=config.n_fft)[:, : config.num_range_bins] / config.adc_samples)
    return torch.cat(profiles)


def range_response(config, low, high, count):
    """Float64 responses [bins, count] of count peak positions spread evenly over [low, high]."""
    centers = low + (high - low) * torch.arange(count, dtype=DTYPE) / max(1, count - 1)
    bins = torch.arange(config.num_range_bins, dtype=DTYPE)
    return dirichlet(bins[:, None] - centers[None], config.adc_samples, config.n_fft)[0]
