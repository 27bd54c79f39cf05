"""Float64 Dirichlet kernel of the range FFT and its windows (oracle; test-only).

D(d) = mean_n exp(-2 pi i n d / n_fft), n < samples, with value and derivative;
restates tests/reference/kernel.py:8-57 and dsplat/kernels/common.slang:10-45.
"""

from __future__ import annotations

import math

import torch


def dirichlet(delta: torch.Tensor, samples: int, n_fft: int | None = None):
    """(D(delta), dD/ddelta) in complex128, periodic in n_fft, with a Taylor branch near 0."""
    n_fft = samples if n_fft is None else n_fft
    delta = delta.double()
    x = delta - n_fft * torch.round(delta / n_fft)
    a, b = math.pi * samples / n_fft, math.pi / n_fft
    h = math.pi * (samples - 1) / n_fft
    near = x.abs() < 1e-3
    safe = torch.where(near, torch.ones_like(x), x)
    sa, sb = torch.sin(a * safe), torch.sin(b * safe)
    ratio = sa / (samples * sb)
    slope = (a * torch.cos(a * safe) * sb - b * sa * torch.cos(b * safe)) / (samples * sb.square())
    c2 = (b * b - a * a) / 6
    c4 = (3 * a**4 + 7 * b**4 - 10 * a * a * b * b) / 360
    ratio = torch.where(near, 1 + c2 * x.square() + c4 * x**4, ratio)
    slope = torch.where(near, 2 * c2 * x + 4 * c4 * x**3, slope)
    phase = torch.exp(-1j * h * x)
    return phase * ratio, phase * (slope - 1j * h * ratio)


def windowed(delta, samples, n_fft=None, window="rect", beta=14.0):
    """Kernel of a rect, hann, hamming or kaiser window (periodic Hann/Hamming by shifts)."""
    n_fft = samples if n_fft is None else n_fft
    if window == "rect":
        return dirichlet(delta, samples, n_fft)
    if window == "kaiser":
        delta = delta.double()
        delta = delta - n_fft * torch.round(delta / n_fft)
        taps = torch.kaiser_window(samples, periodic=False, beta=beta, dtype=torch.float64)
        taps = taps / taps.sum()
        value = torch.zeros_like(delta, dtype=torch.complex128)
        derivative = torch.zeros_like(value)
        for n in range(samples):
            factor = -2j * math.pi * n / n_fft
            term = taps[n] * torch.exp(factor * delta)
            value = value + term
            derivative = derivative + factor * term
        return value, derivative
    a, b = (0.5, 0.5) if window == "hann" else (0.54, 0.46)
    shift = n_fft / samples
    k, dk = dirichlet(delta, samples, n_fft)
    km, dkm = dirichlet(delta - shift, samples, n_fft)
    kp, dkp = dirichlet(delta + shift, samples, n_fft)
    w = b / (2 * a)
    return k - w * (km + kp), dk - w * (dkm + dkp)
