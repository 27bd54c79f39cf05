"""Float64 restatement of the reference's hand-derived surfel adjoint (test infrastructure).

The reference's VJP kernel (dsplat/kernels/surfel.slang:227-311, `vjp_bins`) does not
differentiate the rendered profiles by automatic differentiation: per aperture-surfel
pair it forms two sufficient statistics of the upstream profile g,

    Z0 = conj(c) . sum_k conj(D(k - k0)) g_k,   Z1 = conj(c) . sum_k conj(D'(k - k0)) g_k

(c = carrier rotation), from P = n_fft / samples numerator classes: away from the bin
nearest to k0,

    D(d)  = nu(d) / S (cot(pi d / N) + i),
    D'(d) = ((pi / P) q(d) (cot + i) - (pi / N) nu(d) (1 + cot^2)) / S,

with q(d) = exp(-2 i pi d / P), nu = (1 - q) / (2 i) depending on d only modulo P, so
the bins are summed per class as (cot - i) g and (1 + cot^2) g and multiplied by the
class numerators once (surfel.slang:263-289); the nearest bin uses the directly
evaluated kernel (surfel.slang:287-291). The chain rule through range, obliquity and
carrier phase is surfel.slang:293-301. This module evaluates those same formulas in
float64 on the CPU, vectorised over pairs. It is independent of both the CUDA kernels
(which use their own table form and reduction order) and of the oracle's autograd
derivation (`oracle.fmcw.vjp`), so the tests can pin all three against each other.
"""

from __future__ import annotations

import math

import torch

from .kernel import dirichlet

DTYPE = torch.float64


def _scattering(cosine, distance, fresnel_n, lambda_m):
    """Amplitude cos^2 F(cos) lambda / (8 pi r) and its cos-derivative (scattering.slang:16-40)."""
    visible = cosine > 0
    cos = torch.where(visible, cosine, torch.zeros_like(cosine))
    f = torch.ones_like(cos)
    df = torch.zeros_like(cos)
    if fresnel_n > 1:
        root = torch.sqrt(fresnel_n * fresnel_n - 1 + cos * cos)
        f = (root - cos) / (root + cos)
        df = -2 * (root - cos) / (root * (root + cos))
    path = lambda_m / (8 * math.pi * distance)
    amp = torch.where(visible, path * cos * cos * f, torch.zeros_like(cos))
    amp_cos = torch.where(visible, path * (2 * cos * f + cos * cos * df), torch.zeros_like(cos))
    return amp, amp_cos


def _class_sums(k0, upstream, n_fft, samples):
    """Z-statistics before the carrier: g0 = sum conj(D) g, g1 = sum conj(D') g per pair.

    k0 [A, S] in [0, n_fft); upstream [A, K] complex128. Class form of surfel.slang:254-291.
    """
    pad = n_fft // samples
    bins = upstream.shape[1]
    k = torch.arange(bins, dtype=DTYPE)
    nearest = torch.round(k0)
    offset = nearest - k0  # in [-1/2, 1/2]
    lobe = torch.where(nearest == n_fft, torch.zeros_like(nearest), nearest)
    delta = k[None, None, :] - k0[..., None]  # [A, S, K]
    angle = math.pi * delta / n_fft
    cot = torch.cos(angle) / torch.sin(angle)
    is_lobe = k[None, None, :] == lobe[..., None]
    cot = torch.where(is_lobe, torch.zeros_like(cot), cot)
    g = upstream[:, None, :]  # [A, 1, K]
    first = (cot - 1j) * g  # (cot - i) g
    second = (1 + cot * cot) * g
    keep = (~is_lobe).to(DTYPE)
    first = first * keep
    second = second * keep
    cls = (torch.arange(bins) % pad)
    g0 = torch.zeros(k0.shape, dtype=torch.complex128)
    g1 = torch.zeros_like(g0)
    for p in range(pad):
        members = cls == p
        f_sum = first[..., members].sum(-1)
        s_sum = second[..., members].sum(-1)
        d = p - k0  # any member of the class: q and nu have period pad
        q = torch.exp(-2j * math.pi * d / pad)
        nu = (1 - q) / 2j
        g0 = g0 + nu.conj() * f_sum / samples
        g1 = g1 + ((math.pi / pad) * q.conj() * f_sum - (math.pi / n_fft) * nu.conj() * s_sum) / samples
    # nearest bin: the directly evaluated kernel D(offset) = D_S(offset / P), D' = D_S' / P
    value, slope = dirichlet(offset / pad, samples, samples)
    lobe_index = lobe.long().clamp(max=bins - 1)
    in_range = (lobe < bins)
    nearest_g = torch.gather(upstream, 1, lobe_index) if upstream.shape[0] == k0.shape[0] else None
    nearest_g = torch.where(in_range, nearest_g, torch.zeros_like(nearest_g))
    g0 = g0 + value.conj() * nearest_g
    g1 = g1 + slope.conj() * nearest_g / pad
    return g0, g1


def vjp(config, positions, centers, normals, weights, upstream, fresnel_n=0.0, chunk=16):
    """(grad centers [S, 3], grad normals [S, 3], grad weights [S] complex) by the adjoint formulas.

    Gradients of Re(sum conj(upstream) . render), the same quantity `oracle.fmcw.vjp`
    differentiates by autograd; weights' gradient is sum conj(column) g (PyTorch's
    complex convention).
    """
    p_all = torch.as_tensor(positions).to(DTYPE)
    c = torch.as_tensor(centers).to(DTYPE)
    n = torch.as_tensor(normals).to(DTYPE)
    w = torch.as_tensor(weights).to(torch.complex128)
    g_all = torch.as_tensor(upstream).to(torch.complex128)
    n_fft, samples = config.n_fft, config.adc_samples
    k0_per_meter = 1.0 / config.range_bin_spacing_m
    two_over_c = 2.0 / config.c0_m_s
    gc = torch.zeros_like(c)
    gn = torch.zeros_like(n)
    gw = torch.zeros_like(w)
    for start in range(0, len(p_all), chunk):
        rows = slice(start, min(len(p_all), start + chunk))
        d = p_all[rows][:, None, :] - c[None]  # [A, S, 3]
        r = d.norm(dim=-1)
        u = d / r[..., None]
        cosine = (u * n[None]).sum(-1)
        amp, amp_cos = _scattering(cosine, r, fresnel_n, config.lambda_m)
        tau = two_over_c * r
        cycles = config.fc_hz * tau + config.slope_hz_s * tau * (config.adc_start_time_s - 0.5 * tau)
        rot = torch.exp(2j * math.pi * cycles)
        phase_r = 2 * math.pi * two_over_c * (config.fc_hz + config.slope_hz_s * (config.adc_start_time_s - tau))
        k0 = r * k0_per_meter
        k0 = k0 - n_fft * torch.floor(k0 / n_fft)
        g0, g1 = _class_sums(k0, g_all[rows], n_fft, samples)
        z0 = rot.conj() * g0
        z1 = rot.conj() * g1
        cw = w.conj()[None] * z0
        along = (w.conj()[None] * z1).real * k0_per_meter
        grad_r = -cw.real * amp / r + amp * (cw.imag * phase_r - along)
        grad_cos = cw.real * amp_cos
        visible = (cosine > 0).to(DTYPE)
        grad_r = grad_r * visible
        grad_cos = grad_cos * visible
        gc += (-grad_r[..., None] * u + grad_cos[..., None] * (cosine[..., None] * u - n[None]) / r[..., None]).sum(0)
        gn += (grad_cos[..., None] * u).sum(0)
        gw += (amp * z0 * visible).sum(0)
    return gc, gn, gw
