"""Float64 range/Doppler/azimuth scene renderer on the CPU (test infrastructure only).

Restates the reference's composed renderer (dsplat/surfel.py:132-196 Sensor, project,
fresnel_te, render_scene; tests/reference/physics.py:11-25 for the float64 form): each
surfel's coefficient reflectivity sqrt(area) cos^2 F_TE(cos) r^-gamma exp(4 pi i r / lambda)
multiplies its separable spectral atom at its (range, Doppler, azimuth) bin coordinates.
Everything is differentiable by PyTorch autograd in float64; sensor is any object with the
Sensor fields.
"""

from __future__ import annotations

import math

import torch

from .spectral import design


def wavelength(sensor):
    return sensor.wave_speed / sensor.carrier_hz


def project(positions, velocities, sensor, origin=None, array_axis=None):
    """Bin coordinates [S, 3]: range 2 K r N_r / (c f_s), Doppler 2 N_d T_c (v.u) / lambda,
    azimuth N_a d (u.axis) / lambda (dsplat/surfel.py:152-164)."""
    origin = positions.new_zeros(3) if origin is None else origin
    axis = positions.new_tensor([1.0, 0.0, 0.0]) if array_axis is None else array_axis
    offset = positions - origin
    r = offset.norm(dim=-1).clamp(min=1e-9)
    u = offset / r[:, None]
    nr, nd, na = sensor.shape
    lam = wavelength(sensor)
    pitch = lam / 2 if sensor.spacing_m is None else sensor.spacing_m
    return torch.stack([r * 2 * sensor.slope_hz_s * nr / (sensor.wave_speed * sensor.sample_rate_hz),
                        2 * nd * sensor.chirp_interval_s / lam * (velocities * u).sum(-1),
                        na * pitch / lam * (u * axis).sum(-1)], -1)  # fmt: skip


def fresnel_te(cosine, impedance, ambient=1.0):
    """(eta cos - sqrt(1 - eta^2 sin^2)) / (eta cos + ...), -1 (0 if matched) where cos <= 0
    (dsplat/surfel.py:167-176)."""
    eta = impedance / ambient
    safe = torch.where(cosine > 0, cosine, torch.ones_like(cosine))
    root = torch.sqrt(1 - eta**2 * (1 - safe**2) + 0j)
    value = (eta * safe - root) / (eta * safe + root)
    return torch.where(cosine > 0, value, torch.where(eta == 1, 0j, -1 + 0j))


def render_scene(positions, normals, areas, reflectivity, velocities, impedance, sensor, grid, *,
                 origin=None, gamma=1.0):  # fmt: skip
    """Cube [shape] in complex128; grid is a SpectralGrid(sensor.shape, window)."""
    pos = positions.double()
    origin = pos.new_zeros(3) if origin is None else origin.double()
    toward = origin - pos
    r = toward.norm(dim=-1).clamp(min=1e-9)
    n = normals.double() / normals.double().norm(dim=-1, keepdim=True).clamp(min=1e-12)
    cosine = (n * toward / r[:, None]).sum(-1).clamp(min=0)
    coefficient = (reflectivity.to(torch.complex128) * areas.double().sqrt() * cosine**2
                   * fresnel_te(cosine, impedance.to(torch.complex128)) * r ** (-gamma))  # fmt: skip
    coefficient = coefficient * torch.exp(4j * math.pi * r / wavelength(sensor))
    centers = project(pos, velocities.double(), sensor, origin)
    bins = torch.stack(torch.meshgrid(*[torch.arange(s, dtype=torch.float64) for s in grid.shape],
                                      indexing="ij"), -1).reshape(-1, len(grid.shape))  # fmt: skip
    atoms, _ = design(grid, centers, bins)
    return (atoms @ coefficient).reshape(grid.shape)
