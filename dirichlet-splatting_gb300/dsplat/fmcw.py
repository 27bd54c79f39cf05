"""FMCW sensor: chirp configuration, scans and the surfel measurement model.

A linear chirp (carrier fc, bandwidth B) sampled by adc_samples ADC samples and
zero-padded to n_fft gives, per aperture, the positive range bins
data[A, K] = FFT(ADC, n_fft)[:K] / adc_samples. A surfel at range r appears at bin
r / spacing (spacing = c / (2 B pad)) as the Dirichlet kernel of the range FFT times
the chirp phase. FMCWModel is the measurement model of the solver: rendering and
derivatives on the CUDA kernels, streamed least-squares blocks projected onto the
row basis of the range response, seeded aperture subsets, the range gate and the
FFT range table of the spatial search. Behaviour follows the reference's
dsplat/fmcw.py:62-388.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from math import ceil, floor
from typing import NamedTuple

import torch
import torch.nn.functional as F

from . import surfel
from .kernels import search
from .kernels.gemm import project
from .kernels.response import range_response


@dataclass(frozen=True)
class FMCWConfig:
    fc_hz: float = 120e9
    bandwidth_hz: float = 15e9
    adc_samples: int = 128
    sweep_time_s: float = 1e-5
    adc_start_time_s: float = 0.0
    pad_factor: int = 2
    c0_m_s: float = 299792458.0

    @property
    def lambda_m(self):
        return self.c0_m_s / self.fc_hz

    @property
    def slope_hz_s(self):
        return self.bandwidth_hz / self.sweep_time_s

    @property
    def sample_rate_hz(self):
        return self.adc_samples / self.sweep_time_s

    @property
    def n_fft(self):
        return self.adc_samples * self.pad_factor

    @property
    def num_range_bins(self):
        return self.n_fft // 2

    @property
    def range_bin_spacing_m(self):
        return self.c0_m_s / (2 * self.bandwidth_hz * self.pad_factor)

    @property
    def range_resolution_m(self):
        return self.c0_m_s / (2 * self.bandwidth_hz)


@dataclass(frozen=True)
class Scan:
    """Range profiles data [A, K] measured at scan positions [A, 3], metres."""

    data: torch.Tensor
    scan_positions_m: torch.Tensor
    fmcw_config: FMCWConfig


# --- Row basis of the range response ---------------------------------------------------------

PEAKS_PER_BIN = 16  # peak positions per range bin sampled for the response SVD


@dataclass(frozen=True)
class RowBasis:
    """Orthonormal projection of observation rows stored as consecutive aperture blocks."""

    adjoint: torch.Tensor  # complex [rank, bins] = U^H
    interleaved: torch.Tensor  # real [2 rank, 2 bins] acting on (re, im) row pairs

    def reduce(self, values):
        """Complex rows [blocks * bins, ...] to [blocks * rank, ...]."""
        tail = values.shape[1:]
        rows = values.reshape(-1, self.adjoint.shape[1], tail.numel())
        return (self.adjoint @ rows).reshape(-1, *tail)

    def reduce_major(self, rows):
        """Real rows ordered bin by bin, (2 k + part) * blocks + block, in one product."""
        tail = rows.shape[1:]
        flat = rows.reshape(self.interleaved.shape[1], -1)
        return project(self.interleaved, flat).reshape(-1, *tail)


def response_basis(config, low, high, device):
    """Row basis of all peak positions in [low, high] bins, or None when it spans every bin.

    Singular values below eps / 128 of the largest are dropped, so the normal
    equations keep float32 precision. The SVD runs on the host in float64.
    """
    count = max(2 * config.adc_samples, int(PEAKS_PER_BIN * (high - low)) + 1)
    response = range_response(config, low, high, count, device).cpu()
    vectors, values, _ = torch.linalg.svd(response, full_matrices=False)
    rank = int((values > torch.finfo(torch.float32).eps / 128 * values[0]).sum())
    if rank >= config.num_range_bins:
        return None
    adjoint = vectors[:, :rank].mH
    interleaved = torch.zeros((2 * rank, 2 * config.num_range_bins), dtype=torch.float64)
    interleaved[0::2, 0::2] = adjoint.real
    interleaved[0::2, 1::2] = -adjoint.imag
    interleaved[1::2, 0::2] = adjoint.imag
    interleaved[1::2, 1::2] = adjoint.real
    return RowBasis(adjoint.to(device, torch.complex64), interleaved.to(device, torch.float32))


class RangeTable(NamedTuple):
    """FFT-interpolated range correlations of a residual; they only rank proposals."""

    correlation: torch.Tensor  # [apertures, n_fft * oversample, 2]
    norm: torch.Tensor  # [n_fft * oversample]; carries the observed-bin mask
    oversample: int


# --- Measurement model -----------------------------------------------------------------------


@dataclass(frozen=True)
class FMCWModel:
    """Surfels measured by an FMCW scan.

    params = {centers [S, 3], normals [S, 3], areas [S]}; the coefficients are
    reflectivities. prepare returns a copy carrying the row basis of the centers'
    box; block_bases memoizes the narrower bases of aperture blocks.
    """

    scan: Scan
    fresnel_n: float = 0.0  # known refractive index of the surfels; <= 1 for none
    basis: RowBasis | None = None
    bands: tuple | None = None  # host arrays: per-aperture lowest and highest peak bin
    block_bases: dict = field(default_factory=dict, repr=False)

    @property
    def shape(self):
        return tuple(self.scan.data.shape)

    @property
    def size(self):
        return self.scan.data.numel()

    @property
    def apertures(self):
        return self.shape[0]

    @property
    def row_alignment(self):
        """Streamed blocks hold whole aperture profiles."""
        return self.shape[1]

    @property
    def sensor(self):
        """The chirp configuration and the sensor positions [A, 3]."""
        return self.scan.fmcw_config, self.scan.scan_positions_m

    def sample_apertures(self, count, seed):
        """Sorted ids of a seeded set of whole apertures and the model restricted to them.

        The subset keeps sensor, material and the shared row basis, not the
        per-aperture bands. The same seed selects the same apertures as
        sample_rows with count * bins rows.
        """
        order = torch.randperm(self.shape[0], generator=torch.Generator().manual_seed(seed))
        ids = order[: max(1, count)].sort().values.to(self.scan.data.device)
        scan = replace(
            self.scan,
            data=self.scan.data[ids].contiguous(),
            scan_positions_m=self.scan.scan_positions_m[ids].contiguous(),
        )
        return ids, replace(self, scan=scan, bands=None, block_bases={})

    def sample_rows(self, count, seed, device):
        bins = self.shape[1]
        order = torch.randperm(self.shape[0], generator=torch.Generator().manual_seed(seed))
        chosen = order[: max(1, count // bins)].to(device)
        return (chosen[:, None] * bins + torch.arange(bins, device=device)).flatten()

    def prepare(self, specs):
        """This model with the row basis of every center inside the centers' box.

        The band of range bins runs from the nearest to the farthest box point seen by
        any aperture, widened by one bin. Without a finite box, or when the band would
        wrap around the FFT, the basis covers every peak position.
        """
        lower, upper = specs["centers"].lower, specs["centers"].upper
        config, positions = self.sensor
        low, high, bands = 0.0, float(config.n_fft), None
        if lower is not None and upper is not None:
            lo = positions.new_tensor(lower).expand(3)
            hi = positions.new_tensor(upper).expand(3)
            nearest_point = torch.minimum(torch.maximum(positions, lo), hi)
            farthest_point = torch.where((positions - lo).abs() > (positions - hi).abs(), lo, hi)
            spacing = config.range_bin_spacing_m
            near_bins = ((positions - nearest_point).norm(dim=1) / spacing - 1).clamp(min=0)
            far_bins = (positions - farthest_point).norm(dim=1) / spacing + 1
            near, far = float(near_bins.min()), float(far_bins.max())
            if far - near < config.n_fft:
                low, high = near, far
                bands = (near_bins.cpu().numpy(), far_bins.cpu().numpy())
        basis = response_basis(config, low, high, positions.device)
        return replace(self, basis=basis, bands=bands, block_bases={})

    def block_basis(self, rows):
        """Row basis of a block of whole apertures, never larger than the shared one.

        The block's band is the union of its apertures' bands rounded outward to
        whole critical range samples, so few distinct bases arise; they are built from
        host-side bands and never wait on the device.
        """
        if self.bands is None or self.basis is None:
            return self.basis
        bins, step = self.shape[1], self.scan.fmcw_config.pad_factor
        first, last = rows.start // bins, -(-rows.stop // bins)
        key = (
            floor(self.bands[0][first:last].min() / step) * step,
            ceil(self.bands[1][first:last].max() / step) * step,
        )
        if key not in self.block_bases:
            config, positions = self.sensor
            basis = response_basis(config, float(key[0]), float(key[1]), positions.device)
            narrower = basis is not None and len(basis.adjoint) < len(self.basis.adjoint)
            self.block_bases[key] = basis if narrower else self.basis
        return self.block_bases[key]

    def blocks(self, params, target, real, chunk):
        """Least-squares blocks of whole apertures, projected onto the row basis.

        Real blocks are ordered bin by bin so that one product projects them.
        """
        config, positions = self.sensor
        bins = self.shape[1]
        flat = target.flatten()
        for start in range(0, self.size, chunk):
            rows = slice(start, min(start + chunk, self.size))
            basis = self.block_basis(rows)
            if real:
                block = positions[rows.start // bins : rows.stop // bins]
                a = surfel.design(config, block, params, self.fresnel_n, real=True)
                y = torch.view_as_real(flat[rows]).reshape(len(block), 2 * bins).T.reshape(-1)
                yield (a, y) if basis is None else (basis.reduce_major(a), basis.reduce_major(y))
            else:
                a, y = self.design(params, rows), flat[rows]
                yield (a, y) if basis is None else (basis.reduce(a), basis.reduce(y))

    def _apertures(self, rows):
        """Apertures of arbitrary row ids, each row's index among them, and its bin."""
        apertures, inverse = torch.unique(rows // self.shape[1], return_inverse=True)
        return self.scan.scan_positions_m[apertures], inverse, rows % self.shape[1]

    def design(self, params, rows):
        """Complex dictionary rows [rows, S]; a slice must cover whole apertures."""
        config, positions = self.sensor
        bins = self.shape[1]
        if isinstance(rows, slice):
            block = positions[rows.start // bins : -(-rows.stop // bins)]
            return surfel.design(config, block, params, self.fresnel_n)
        block, inverse, ids = self._apertures(rows)
        a = surfel.design(config, block, params, self.fresnel_n)
        return a.reshape(len(block), bins, -1)[inverse, ids]

    def jacobian(self, params, rows, atoms, keys):
        """Column derivatives [rows, atoms, D] for the given parameter keys and row ids."""
        block, inverse, ids = self._apertures(rows)
        selected = {key: value[atoms] for key, value in params.items()}
        derivatives = surfel.jacobian(self.scan.fmcw_config, block, selected, self.fresnel_n)
        return {key: derivatives[key][inverse, ids] for key in keys}

    def render(self, params, coefficients):
        return surfel.render(*self.sensor, params, coefficients, self.fresnel_n)

    def jvp(self, params, coefficients, tangent, delta_coefficients):
        return surfel.jvp(
            *self.sensor, params, coefficients, tangent, delta_coefficients, self.fresnel_n
        )

    def vjp(self, params, coefficients, upstream):
        return surfel.vjp(*self.sensor, params, coefficients, upstream, self.fresnel_n)

    def correlate(self, params, residual, active=None):
        return surfel.correlate(*self.sensor, params, residual.reshape(self.shape), self.fresnel_n, active)

    def correlate_gradient(self, params, residual, include_normals=False):
        return surfel.correlate_gradient(
            *self.sensor, params, residual.reshape(self.shape), self.fresnel_n, include_normals
        )

    def correlate_orientations(self, params, residual, bank, table=None):
        return surfel.correlate_orientations(
            *self.sensor, params, bank, residual.reshape(self.shape), self.fresnel_n, table
        )

    @torch.no_grad()
    def range_gate(self, points, measurement, relative_power, margin_cells, min_fraction):
        """Points whose spherical range falls in a measured range interval at enough apertures.

        32 evenly spaced apertures threshold their profile relative to its own peak,
        dilate every interval above it by margin_cells range resolutions, and a point
        must hit an interval at min_fraction of the apertures with signal.
        """
        config, positions = self.sensor
        count = min(32, len(measurement))
        ids = torch.linspace(0, len(measurement) - 1, count, device=points.device).long()
        power = measurement[ids].abs().square()
        peak = power.max(-1).values
        informative = peak > peak.max() * 1e-6
        power, peak = power[informative], peak[informative]
        spacing = config.range_bin_spacing_m
        radius = math.ceil(margin_cells * config.range_resolution_m / spacing)
        above = (power >= relative_power * peak[:, None]).float()[:, None]
        intervals = F.max_pool1d(above, 2 * radius + 1, stride=1, padding=radius)[:, 0].int()
        return search.range_gate(points, positions[ids][informative], intervals, spacing, min_fraction)

    @torch.no_grad()
    def range_table(self, residual, oversample=8):
        """Oversampled FFT range correlations of the residual for proposal scores."""
        config = self.scan.fmcw_config
        n, samples = config.n_fft, config.adc_samples
        size = n * oversample
        residual = residual.reshape(self.shape)
        coefficients = torch.fft.ifft(residual, n=n, dim=-1)[..., :samples] * (n / samples)
        correlation = torch.fft.fft(coefficients, n=size, dim=-1)
        kernel = torch.fft.fft(residual.real.new_ones(samples), n=size) / samples
        mask = residual.real.new_zeros(size)
        mask[: config.num_range_bins * oversample : oversample] = 1
        norm = torch.fft.ifft(torch.fft.fft(mask) * torch.fft.fft(kernel.abs().square())).real
        return RangeTable(torch.view_as_real(correlation).contiguous(), norm.contiguous(), oversample)


# --- Initialization ---------------------------------------------------------------------


@torch.no_grad()
def migration(scan, points, aperture_shape, *, depth_samples=96, padding=2, frequency_chunk=16):
    """Relative complex focusing strength of a planar raster scan at world-space points.

    Reference: dsplat/fmcw.py:361-454. The scan must be a complete row-major planar raster
    and the points lie on one side of it. The positive range bins are zero-filled back to
    chirp samples with the residual-video-phase correction, every ADC sample's aperture
    field is propagated by the angular spectrum (K = 4 pi f / c, every propagating replica
    of an undersampled aperture kept), and the focused volume is interpolated at the
    points. A scalar Green model without obliquity or Fresnel factors: an initializer,
    not a calibrated reflectivity. The frequency sum of every (depth, kx, ky) runs in one
    CUDA kernel (dsg_migration_focus); frequency_chunk is accepted for the reference's
    signature and has no effect.
    """
    from .kernels import _lib

    del frequency_chunk
    nu, nv = aperture_shape
    raster = scan.scan_positions_m.reshape(nu, nv, 3)
    center = raster[nu // 2, nv // 2]
    step_u = (raster[-1, 0] - raster[0, 0]) / (nu - 1)
    step_v = (raster[0, -1] - raster[0, 0]) / (nv - 1)
    du, dv = float(step_u.norm()), float(step_v.norm())
    eu, ev = step_u / du, step_v / dv
    local = (points - center) @ torch.stack([eu, ev, torch.linalg.cross(eu, ev)], -1)
    local[:, 2] = local[:, 2].abs()
    z_low, z_high = local[:, 2].min(), local[:, 2].max()
    if float(z_high - z_low) < 1e-6:
        depth_samples = 1
    cfg = scan.fmcw_config
    device, dtype = points.device, points.dtype
    # back to chirp samples: undo the residual video phase, inverse range FFT
    beat_hz = torch.arange(cfg.num_range_bins, device=device, dtype=dtype) * (cfg.sample_rate_hz / cfg.n_fft)
    video = scan.data * torch.exp(1j * math.pi * beat_hz.square() / cfg.slope_hz_s)
    adc = torch.fft.ifft(video, n=cfg.n_fft, dim=-1)[..., : cfg.adc_samples] * cfg.adc_samples
    pu, pv = nu * padding, nv * padding
    field = adc.new_zeros((cfg.adc_samples, pu, pv))
    ou, ov = pu // 2 - nu // 2, pv // 2 - nv // 2
    field[:, ou : ou + nu, ov : ov + nv] = adc.reshape(nu, nv, -1).permute(2, 0, 1)
    spectrum = torch.fft.fftshift(torch.fft.fft2(torch.fft.ifftshift(field, dim=(-2, -1))), dim=(-2, -1))
    times = cfg.adc_start_time_s + torch.arange(cfg.adc_samples, device=device, dtype=dtype) / cfg.sample_rate_hz
    wavenumber = 4 * math.pi * (cfg.fc_hz + cfg.slope_hz_s * times) / cfg.c0_m_s
    carrier = wavenumber.max() / 2
    planes = torch.unique(local[:, 2])
    uniform = len(planes) < 3 or torch.allclose(
        planes.diff(), planes.diff().mean().expand(len(planes) - 1), atol=1e-7, rtol=1e-4
    )
    if len(planes) <= depth_samples and uniform:
        depths = planes  # the points already lie on these regularly spaced planes
    else:
        # |kz - carrier| <= Kmax / 2: four samples per Nyquist interval in depth
        count = max(depth_samples, 1 + math.ceil(float(z_high - z_low) * float(wavenumber.max()) * 2 / math.pi))
        depths = torch.linspace(float(z_low), float(z_high), count, device=device, dtype=dtype)
    # every propagating replica of the sampled aperture spectrum
    copies_u = max(1, math.ceil(float(wavenumber.max()) * du / math.pi))
    copies_v = max(1, math.ceil(float(wavenumber.max()) * dv / math.pi))
    qu, qv = pu * copies_u, pv * copies_v
    dx, dy = du / copies_u, dv / copies_v
    kx = 2 * math.pi * torch.fft.fftshift(torch.fft.fftfreq(qu, d=dx, device=device, dtype=dtype))
    ky = 2 * math.pi * torch.fft.fftshift(torch.fft.fftfreq(qv, d=dy, device=device, dtype=dtype))
    spectrum_c = torch.view_as_real(spectrum.to(torch.complex64).contiguous()).contiguous()
    depth32 = depths.to(torch.float32).contiguous()
    focused = torch.empty((len(depths), qu, qv, 2), dtype=torch.float32, device=device)
    _lib.call(
        "dsg_migration_focus", _lib.ptr(spectrum_c), cfg.adc_samples, pu, pv,
        _lib.ptr(wavenumber.to(torch.float32).contiguous()), _lib.ptr(kx.to(torch.float32).contiguous()),
        _lib.ptr(ky.to(torch.float32).contiguous()), qu, qv, _lib.ptr(depth32), len(depths), _lib.ptr(focused),
        _lib.stream(device),
    )  # fmt: skip
    pitch = local.new_tensor([dx, dy])
    low = torch.floor(local[:, :2].min(0).values / pitch).long() - 2
    high = torch.ceil(local[:, :2].max(0).values / pitch).long() + 2
    a, b = int(low[0]) + qu // 2, int(high[0]) + qu // 2 + 1
    c, d = int(low[1]) + qv // 2, int(high[1]) + qv // 2 + 1
    planes_xy = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(torch.view_as_complex(focused), dim=(-2, -1))),
                                   dim=(-2, -1))  # fmt: skip
    # remove the carrier before interpolating (the band is then centred), restore it after
    volume = planes_xy[:, a:b, c:d] * torch.exp(1j * carrier * depths)[:, None, None]
    volume = volume * (copies_u * copies_v / cfg.adc_samples)
    xy = 2 * (local[:, :2] - low * pitch) / ((high - low) * pitch) - 1
    zz = 2 * (local[:, 2] - z_low) / (z_high - z_low) - 1 if len(depths) > 1 else torch.zeros_like(local[:, 2])
    where = torch.stack([xy[:, 1], xy[:, 0], zz], -1).reshape(1, 1, 1, -1, 3)
    channels = torch.view_as_real(volume).permute(3, 0, 1, 2)[None]
    sampled = F.grid_sample(channels, where, mode="bilinear", align_corners=True).reshape(2, -1)
    return torch.complex(sampled[0], sampled[1]) * torch.exp(-1j * carrier * local[:, 2])
