"""Synthetic ground truth: planar arrays and FMCW scans of known surfels.

synthesize follows the FMCW signal chain itself: each surfel echo is a beat tone
sampled by the ADC, summed in double precision and range-FFT'd; it never evaluates
the Dirichlet kernel, so a fit to its scans does not reuse the forward model
(reference: dsplat/groundtruth.py:16-90).
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .fmcw import Scan


def planar_array(side, pitch, axis=(0.0, 0.0, 1.0), standoff=0.35, *, device="cpu"):
    """side x side aperture positions [side^2, 3] in metres, pitch apart.

    The array faces along axis toward (0, 0, standoff); the default is the plane
    z = 0 facing +z. The rotation takes +z to axis (Rodrigues' formula).
    """
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    zhat = np.array([0.0, 0.0, 1.0])
    k = np.cross(zhat, axis)
    cos = float(zhat @ axis)
    if np.linalg.norm(k) < 1e-10:
        rotation = np.eye(3) if cos > 0 else np.diag([1.0, -1.0, -1.0])
    else:
        skew = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        rotation = np.eye(3) + skew + skew @ skew / (1 + cos)
    t = (np.arange(side) - (side - 1) / 2) * pitch
    gx, gy = np.meshgrid(t, t, indexing="ij")
    flat = np.stack([gx.ravel(), gy.ravel(), np.zeros(side * side)], -1)
    center = np.array([0.0, 0.0, standoff])
    return torch.tensor(center + (flat - center) @ rotation.T, dtype=torch.float32, device=device)


def _echoes(aperture_positions, surfel_centers, surfel_normals, config, fresnel_n=0.0):
    """Range [A, S] and complex echo amplitude [A, S] of each aperture-surfel pair."""
    diff = aperture_positions[:, None, :] - surfel_centers[None, :, :]
    distance = diff.norm(dim=-1).clamp(min=1e-9)
    cosine = (diff / distance[..., None] * surfel_normals[None]).sum(-1).clamp(min=0)
    amplitude = cosine.square() * config.lambda_m / (8 * math.pi * distance)
    if fresnel_n > 1:
        root = torch.sqrt(fresnel_n * fresnel_n - 1 + cosine.square())
        amplitude = amplitude * (root - cosine) / (root + cosine)
    tau = 2 * distance / config.c0_m_s
    cycles = config.fc_hz * tau + config.slope_hz_s * tau * (config.adc_start_time_s - 0.5 * tau)
    return distance, amplitude * torch.exp(2j * math.pi * cycles)


@torch.no_grad()
def synthesize(aperture_positions, surfel_centers, surfel_normals, surfel_amplitudes, config,
               fresnel_n=0.0):  # fmt: skip
    """Scan [apertures, range bins] of surfels with amplitudes reflectivity * sqrt(area).

    The ADC samples are summed in float64 by dsg_synthesize_adc on the surfels' device;
    the range FFT is torch.fft. Inputs must be CUDA tensors.
    """
    from .kernels import _lib

    device = surfel_centers.device
    positions = aperture_positions.to(device=device, dtype=torch.float64).contiguous()
    centers = surfel_centers.to(torch.float64).contiguous()
    normals = surfel_normals.to(torch.float64).contiguous()
    amplitudes = torch.view_as_real(surfel_amplitudes.to(torch.complex128).reshape(-1).contiguous())
    adc = torch.empty((len(positions), config.adc_samples, 2), dtype=torch.float64, device=device)
    _lib.call(
        "dsg_synthesize_adc", _lib.chirp(config, fresnel_n), float(config.sample_rate_hz), _lib.ptr(positions),
        len(positions), _lib.ptr(centers), _lib.ptr(normals), _lib.ptr(amplitudes), len(centers), _lib.ptr(adc),
        _lib.stream(device),
    )  # fmt: skip
    spectrum = torch.fft.fft(torch.view_as_complex(adc), n=config.n_fft)[:, : config.num_range_bins]
    return Scan((spectrum / config.adc_samples).to(torch.complex64), aperture_positions, config)
