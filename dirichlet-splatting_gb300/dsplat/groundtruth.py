"""Synthetic ground truth: planar arrays and FMCW scans of known surfels.

synthesize follows the FMCW signal chain itself: every surfel's echo is a beat tone
sampled by the ADC, the samples are summed in float64 on the GPU (dsg_synthesize_adc)
and range-FFT'd. It never evaluates the Dirichlet kernel, so a fit to its scans does not
reuse the forward model. Behaviour of the reference's dsplat/groundtruth.py:16-90.
"""

from __future__ import annotations

import torch

from .fmcw import Scan


def _rotation_from_z(axis):
    """The 3 x 3 float64 rotation taking +z onto the unit vector axis.

    Rodrigues' form I + [k]x + [k]x^2 / (1 + cos) with k = z x axis; the antiparallel
    case, where that form is undefined, is the half turn about x.
    """
    a = torch.as_tensor(axis, dtype=torch.float64)
    a = a / a.norm()
    z = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64)
    k = torch.linalg.cross(z, a)
    cos = float(z @ a)
    if float(k.norm()) < 1e-10:
        flip = torch.tensor([1.0, -1.0, -1.0], dtype=torch.float64)
        return torch.eye(3, dtype=torch.float64) if cos > 0 else torch.diag(flip)
    skew = torch.zeros(3, 3, dtype=torch.float64)
    skew[0, 1], skew[0, 2], skew[1, 2] = -k[2], k[1], -k[0]
    skew = skew - skew.T
    return torch.eye(3, dtype=torch.float64) + skew + skew @ skew / (1 + cos)


def planar_array(side, pitch, axis=(0.0, 0.0, 1.0), standoff=0.35, *, device="cpu"):
    """side x side aperture positions [side^2, 3] in metres, pitch apart, row-major.

    The array lies in z = 0 facing +z, then turns about (0, 0, standoff) so that it
    faces along axis.
    """
    offsets = (torch.arange(side, dtype=torch.float64) - (side - 1) / 2) * pitch
    flat = torch.cartesian_prod(offsets, offsets)
    plane = torch.cat((flat, torch.zeros(side * side, 1, dtype=torch.float64)), 1)
    pivot = torch.tensor([0.0, 0.0, standoff], dtype=torch.float64)
    turned = pivot + (plane - pivot) @ _rotation_from_z(axis).T
    return turned.to(device=device, dtype=torch.float32)


@torch.no_grad()
def synthesize(aperture_positions, surfel_centers, surfel_normals, surfel_amplitudes, config, fresnel_n=0.0):
    """Scan [apertures, range bins] of surfels with amplitudes reflectivity * sqrt(area).

    The echoes' ADC samples are summed in float64 by dsg_synthesize_adc on the surfels'
    device (CUDA tensors only); the range FFT is torch.fft, scaled by 1 / adc_samples.
    """
    from .kernels import _lib

    device = surfel_centers.device
    # every buffer the kernel reads stays referenced here until the launch is queued
    positions = aperture_positions.to(device=device, dtype=torch.float64).contiguous()
    centers = surfel_centers.to(torch.float64).contiguous()
    normals = surfel_normals.to(torch.float64).contiguous()
    amplitudes = torch.view_as_real(surfel_amplitudes.to(torch.complex128).reshape(-1).contiguous())
    adc = torch.empty((len(positions), config.adc_samples, 2), device=device, dtype=torch.float64)
    _lib.call("dsg_synthesize_adc", _lib.chirp(config, fresnel_n), float(config.sample_rate_hz), _lib.ptr(positions),
              len(positions), _lib.ptr(centers), _lib.ptr(normals), _lib.ptr(amplitudes), len(centers),
              _lib.ptr(adc), _lib.stream(device))  # fmt: skip
    bins = torch.fft.fft(torch.view_as_complex(adc), n=config.n_fft)[:, : config.num_range_bins]
    return Scan((bins / config.adc_samples).to(torch.complex64), aperture_positions, config)
