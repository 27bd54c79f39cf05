"""Oriented surfels, the scattering primitive of the FMCW measurements.

A surfel has a center [3] (m), an outward unit normal [3] and an area (m^2); its
reflectivity b is the linear coefficient variable projection solves, its material a
known refractive index fresnel_n (<= 1 for none). Seen from a monostatic sensor at
p, with r = |p - c|, u = (p - c) / r and cos = u . n:

    amplitude = sqrt(area) cos^2 F(cos) lambda / (8 pi r)     zero when cos <= 0
    F(cos)    = (root - cos) / (root + cos),  root = sqrt(fresnel_n^2 - 1 + cos^2)
    delay     = 2 r / c

The echo depends on area and reflectivity only through w = b sqrt(area). These
functions carry that area chain around the CUDA kernels of dsplat.kernels.surfel
(reference: dsplat/surfel.py:45-129).
"""

from __future__ import annotations

from dataclasses import dataclass

import torch

from .kernels import surfel as kernel


def render(config, positions, params, coefficients, fresnel_n=0.0):
    """Range profiles [A, K] of surfels with reflectivities coefficients; differentiable."""
    weights = coefficients * params["areas"].sqrt()
    return kernel.render(config, positions, params["centers"], params["normals"], weights, fresnel_n)


def jvp(config, positions, params, coefficients, tangent, delta_coefficients, fresnel_n=0.0):
    """Change of the profiles along tangent (centers, normals, areas) and delta_coefficients.

    With s = sqrt(area): dw = db s + b d(area) / (2 s).
    """
    root = params["areas"].sqrt()
    weights = coefficients * root
    delta_weights = delta_coefficients * root + coefficients * tangent["areas"] / (2 * root)
    return kernel.jvp(
        config, positions, params["centers"], params["normals"], weights,
        tangent["centers"], tangent["normals"], delta_weights, fresnel_n,
    )  # fmt: skip


def vjp(config, positions, params, coefficients, upstream, fresnel_n=0.0):
    """Gradients of Re(conj(upstream) . profiles) per parameter and for the coefficients."""
    root = params["areas"].sqrt()
    centers, normals, grad_weights = kernel.vjp(
        config, positions, params["centers"], params["normals"], coefficients * root, upstream,
        fresnel_n,
    )  # fmt: skip
    areas = (grad_weights.conj() * coefficients).real / (2 * root)
    return dict(centers=centers, normals=normals, areas=areas), grad_weights * root


def design(config, positions, params, fresnel_n=0.0, real=False):
    """Dictionary columns of every surfel for whole apertures; see kernels.surfel.design."""
    return kernel.design(
        config, positions, params["centers"], params["normals"], params["areas"], fresnel_n, real
    )


def jacobian(config, positions, params, fresnel_n=0.0):
    """Derivatives of the columns [A, K, S] by centers and normals [..., 3] and areas [..., 1]."""
    columns, dc, dn = kernel.jacobian(config, positions, params["centers"], params["normals"], fresnel_n)
    root = params["areas"].sqrt()
    return {
        "centers": dc * root[:, None],
        "normals": dn * root[:, None],
        "areas": (columns / (2 * root))[..., None],
    }


def correlate(config, positions, params, residual, fresnel_n=0.0, active=None):
    """a^H r and |a|^2 of every surfel's column a against the residual profiles [A, K].

    active (count tensor, period) restricts the work to surfels whose index mod period is
    below count (the others return zeros).
    """
    corr, norm = kernel.correlate(
        config, positions, params["centers"], params["normals"], residual, fresnel_n, active
    )
    return corr * params["areas"].sqrt(), norm * params["areas"]


def correlate_gradient(config, positions, params, residual, fresnel_n=0.0, include_normals=False):
    """correlate and its derivatives by centers (and normals): corr, norm, dcorr, dnorm."""
    corr, norm, dcorr, dnorm = kernel.correlate_gradient(
        config, positions, params["centers"], params["normals"], residual, fresnel_n,
        include_normals,
    )  # fmt: skip
    root, area = params["areas"].sqrt(), params["areas"]
    return corr * root, norm * area, dcorr * root[:, None], dnorm * area[:, None]


def correlate_orientations(config, positions, params, bank, residual, fresnel_n=0.0, table=None):
    """correlate for each surfel's own normal and every bank normal, [S, 1 + bank]."""
    corr, norm = kernel.correlate_orientations(
        config, positions, params["centers"], params["normals"], bank, residual, fresnel_n, table
    )
    root = params["areas"].sqrt()[:, None]
    return corr * root, norm * root.square()


def orient_best(config, positions, params, bank, residual, energy, real_mode, fresnel_n=0.0, table=None):
    """(which, top): each surfel's best normal among its own and the bank's, and its certificate."""
    return kernel.orient_best(config, positions, params["centers"], params["normals"], params["areas"], bank,
                              residual, fresnel_n, energy, real_mode, table)  # fmt: skip


# --- Range / Doppler / azimuth composition (13 degrees of freedom per surfel) ----------------
# Reference: dsplat/surfel.py:132-196. A surfel has position [3], normal [3], area,
# complex reflectivity, velocity [3] and complex material impedance; a monostatic
# range/Doppler/azimuth sensor maps it to a point of a separable spectral grid, where the
# spectral kernels (dsplat.kernels.spectral) render it. Gradients reach all thirteen
# quantities through autograd and the hand-written spectral VJP.


@dataclass(frozen=True)
class Sensor:
    """A range/Doppler/azimuth sensor: bins per axis and the chirp constants."""

    shape: tuple[int, int, int] = (128, 32, 16)  # range, Doppler, azimuth bins
    carrier_hz: float = 77e9
    sample_rate_hz: float = 2e6
    slope_hz_s: float = 20e12
    chirp_interval_s: float = 60e-6
    spacing_m: float | None = None  # array pitch; None: half a wavelength
    wave_speed: float = 299792458.0

    @property
    def wavelength(self):
        return self.wave_speed / self.carrier_hz


def project(positions, velocities, sensor: Sensor, origin=None, array_axis=None):
    """Fractional (range, Doppler, azimuth) bin coordinates [S, 3] of moving points.

    range bin = 2 K r N_r / (c f_s); Doppler bin = 2 N_d T_c (v . u) / lambda; azimuth
    bin = N_a d (u . axis) / lambda, with u the unit line of sight from the origin.
    """
    origin = positions.new_zeros(3) if origin is None else origin
    axis = positions.new_tensor([1.0, 0.0, 0.0]) if array_axis is None else array_axis
    offset = positions - origin
    distance = offset.norm(dim=-1).clamp(min=1e-9)
    sight = offset / distance[:, None]
    n_range, n_doppler, n_azimuth = sensor.shape
    pitch = sensor.wavelength / 2 if sensor.spacing_m is None else sensor.spacing_m
    range_bin = distance * (2 * sensor.slope_hz_s / sensor.wave_speed * n_range / sensor.sample_rate_hz)
    doppler_bin = (velocities * sight).sum(-1) * (2 * n_doppler * sensor.chirp_interval_s / sensor.wavelength)
    azimuth_bin = (sight * axis).sum(-1) * (n_azimuth * pitch / sensor.wavelength)
    return torch.stack([range_bin, doppler_bin, azimuth_bin], -1)


def fresnel_te(cosine, impedance, ambient=1.0):
    """TE reflection coefficient of a material with complex impedance (0 gives -1).

    Where cos <= 0 the amplitude vanishes anyway; the coefficient is then -1, or 0 for a
    matched interface, and is evaluated at a harmless cosine so no NaN reaches autograd.
    """
    eta = impedance / ambient
    safe = torch.where(cosine > 0, cosine, torch.ones_like(cosine))
    transmitted = torch.sqrt(1 - eta.square() * (1 - safe.square()) + 0j)
    coefficient = (eta * safe - transmitted) / (eta * safe + transmitted)
    outside = torch.where(eta == 1, torch.zeros_like(coefficient), -torch.ones_like(coefficient))
    return torch.where(cosine > 0, coefficient, outside)


def render_scene(positions, normals, areas, reflectivity, velocities, impedance, sensor: Sensor, *,
                 origin=None, gamma=1.0, window="rect"):  # fmt: skip
    """Coherent range/Doppler/azimuth cube of 13-DOF surfels; differentiable in all of them.

    coefficient = reflectivity sqrt(area) cos^2 F_TE(cos) r^-gamma exp(4 pi i r / lambda),
    placed at project(...) on a SpectralGrid(sensor.shape, window) and rendered by the
    spectral kernel.
    """
    from .kernels import spectral as spectral_kernel
    from .spectral import SpectralGrid

    origin = positions.new_zeros(3) if origin is None else origin
    toward = origin - positions
    distance = toward.norm(dim=-1).clamp(min=1e-9)
    unit = torch.nn.functional.normalize(normals, dim=-1)
    cosine = (unit * toward / distance[:, None]).sum(-1).clamp(min=0)
    coefficient = (reflectivity * areas.sqrt() * cosine.square() * fresnel_te(cosine, impedance)
                   * distance.pow(-gamma))  # fmt: skip
    coefficient = coefficient * torch.exp(4j * torch.pi * distance / sensor.wavelength)
    grid = SpectralGrid(sensor.shape, window=window)
    centers = project(positions, velocities, sensor, origin)
    return spectral_kernel.render(grid, centers, coefficient, grid.bins(positions.device)).reshape(grid.shape)
