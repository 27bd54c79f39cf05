"""FMCW sensor: chirp constants, scans and the surfel measurement model.

A linear chirp (carrier fc, bandwidth B) sampled by adc_samples ADC samples and
zero-padded to n_fft gives, per aperture, the positive range bins
data[A, K] = FFT(ADC, n_fft)[:K] / adc_samples. A surfel at range r shows up at bin
r / spacing (spacing = c / (2 B pad)) as the Dirichlet kernel of the range FFT times
its carrier phase.

FMCWModel is the solver's measurement model. Rendering and derivatives run on the CUDA
kernels (dsplat.surfel -> libdsplat_gb300.so); least-squares rows are streamed in whole
aperture blocks and projected onto an orthonormal basis of the range responses that
the fit's box can produce (a rank r << K subspace per block, from a float64 SVD on
the host); aperture subsets are drawn from a seeded CPU generator so they match the
reference's draws. Behaviour: the reference's dsplat/fmcw.py:29-454.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
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


# --- Row basis of the range responses --------------------------------------------------------

RESPONSE_SAMPLES_PER_BIN = 16  # peak positions per range bin in the sampled response matrix


@dataclass(frozen=True)
class RowBasis:
    """An orthonormal projection U^H of the rows of consecutive aperture blocks."""

    adjoint: torch.Tensor  # complex [rank, bins] = U^H
    interleaved: torch.Tensor  # real [2 rank, 2 bins]: U^H acting on (re, im) pairs

    def reduce(self, values):
        """Complex rows [blocks * bins, ...] -> [blocks * rank, ...]."""
        bins = self.adjoint.shape[1]
        tail = values.shape[1:]
        stacked = values.reshape(-1, bins, tail.numel())
        return torch.matmul(self.adjoint, stacked).reshape(-1, *tail)

    def reduce_major(self, rows):
        """Real rows in bin-major order ((2 k + part) * blocks + block) reduced in one product."""
        tail = rows.shape[1:]
        return project(self.interleaved, rows.reshape(self.interleaved.shape[1], -1)).reshape(-1, *tail)


def _interleave(adjoint):
    """The real [2 r, 2 K] matrix of a complex [r, K] one acting on (re, im) pairs."""
    r, k = adjoint.shape
    re, im = adjoint.real, adjoint.imag
    blocks = torch.stack((torch.stack((re, -im), -1), torch.stack((im, re), -1)), 1)  # [r, 2, K, 2]
    return blocks.reshape(2 * r, 2 * k)


def response_basis(config, low, high, device):
    """Row basis of every peak position in [low, high] bins, or None if it needs every bin.

    The range responses of peaks spread over the band span a subspace of low numerical
    rank; singular directions below eps / 128 of the largest are dropped (the normal
    equations then keep float32 accuracy). The SVD runs on the host in float64.
    """
    count = max(2 * config.adc_samples, int(RESPONSE_SAMPLES_PER_BIN * (high - low)) + 1)
    response = range_response(config, low, high, count, device).cpu()
    left, sigma, _ = torch.linalg.svd(response, full_matrices=False)
    keep = int((sigma > sigma[0] * (torch.finfo(torch.float32).eps / 128)).sum())
    if keep >= config.num_range_bins:
        return None
    adjoint = left[:, :keep].mH
    return RowBasis(adjoint.to(device, torch.complex64), _interleave(adjoint).to(device, torch.float32))


class RangeTable(NamedTuple):
    """FFT-interpolated range correlations of a residual; used to rank proposals only."""

    correlation: torch.Tensor  # [apertures, n_fft * oversample, 2]
    norm: torch.Tensor  # [n_fft * oversample], carrying the observed-bin mask
    oversample: int


# --- Measurement model -----------------------------------------------------------------------


def _seeded_order(count, seed):
    """The aperture order of a seeded CPU generator (the same draws as the reference)."""
    return torch.randperm(count, generator=torch.Generator().manual_seed(seed))


@dataclass(frozen=True)
class FMCWModel:
    """Surfels {centers [S, 3], normals [S, 3], areas [S]} seen by an FMCW scan.

    The coefficients are reflectivities. prepare() returns a copy carrying the row basis
    of the centers' box and per-aperture bands; block_basis memoizes the narrower bases
    of aperture blocks by their band.
    """

    scan: Scan
    fresnel_n: float = 0.0  # known refractive index of the surfels; <= 1 for none
    basis: RowBasis | None = None
    bands: tuple | None = None  # host arrays: per-aperture nearest and farthest box bin
    block_bases: dict = field(default_factory=dict, repr=False)

    # -- shape ---------------------------------------------------------------------------------

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
        """(chirp configuration, sensor positions [A, 3])."""
        return self.scan.fmcw_config, self.scan.scan_positions_m

    # -- subsets ---------------------------------------------------------------------------------

    def sample_apertures(self, count, seed):
        """Sorted ids of count seeded apertures and this model restricted to them.

        The subset keeps the sensor, the material and the shared row basis, not the
        per-aperture bands; the same seed picks the apertures sample_rows picks.
        """
        picked = _seeded_order(self.apertures, seed)[: max(1, count)]
        ids = torch.sort(picked).values.to(self.scan.data.device)
        sub = Scan(self.scan.data[ids].contiguous(), self.scan.scan_positions_m[ids].contiguous(),
                   self.scan.fmcw_config)  # fmt: skip
        return ids, replace(self, scan=sub, bands=None, block_bases={})

    def sample_rows(self, count, seed, device):
        """Row ids of the whole profiles of count // bins seeded apertures (in draw order)."""
        bins = self.shape[1]
        picked = _seeded_order(self.apertures, seed)[: max(1, count // bins)].to(device)
        return (picked[:, None] * bins + torch.arange(bins, device=device)[None]).reshape(-1)

    # -- row bases -------------------------------------------------------------------------------

    def prepare(self, specs):
        """This model with the row basis of every center inside the centers' box.

        Each aperture's band runs from its nearest to its farthest box point, widened by
        one bin; the shared band covers all apertures. Without a finite box, or when the
        band would wrap around the FFT, the basis covers every peak position.
        """
        config, positions = self.sensor
        low, high, bands = 0.0, float(config.n_fft), None
        lower, upper = specs["centers"].lower, specs["centers"].upper
        if lower is not None and upper is not None:
            box_low = positions.new_tensor(lower).expand(3)
            box_high = positions.new_tensor(upper).expand(3)
            closest = positions.clamp(min=box_low, max=box_high)
            farthest = torch.where((positions - box_low).abs() > (positions - box_high).abs(), box_low, box_high)
            per_bin = 1.0 / config.range_bin_spacing_m
            near = ((positions - closest).norm(dim=1) * per_bin - 1).clamp(min=0)
            far = (positions - farthest).norm(dim=1) * per_bin + 1
            span = torch.stack((near.min(), far.max())).tolist()
            if span[1] - span[0] < config.n_fft:
                low, high = span
                bands = (near.cpu().numpy(), far.cpu().numpy())
        basis = response_basis(config, low, high, positions.device)
        return replace(self, basis=basis, bands=bands, block_bases={})

    def block_basis(self, rows):
        """Row basis of a block of whole apertures, never wider than the shared one.

        The block's band is the union of its apertures' bands rounded outward to whole
        multiples of the pad factor (critical range samples), so few distinct bases exist;
        they come from host-side bands and never wait on the device.
        """
        if self.bands is None or self.basis is None:
            return self.basis
        bins, step = self.shape[1], self.scan.fmcw_config.pad_factor
        first, stop = rows.start // bins, -(-rows.stop // bins)
        near, far = self.bands[0][first:stop].min(), self.bands[1][first:stop].max()
        band = (math.floor(near / step) * step, math.ceil(far / step) * step)
        basis = self.block_bases.get(band)
        if basis is None:
            config, positions = self.sensor
            own = response_basis(config, float(band[0]), float(band[1]), positions.device)
            basis = own if own is not None and own.adjoint.shape[0] < self.basis.adjoint.shape[0] else self.basis
            self.block_bases[band] = basis
        return basis

    def blocks(self, params, target, real, chunk):
        """Projected least-squares blocks (rows a, data y) of whole apertures.

        Real blocks are bin-major, so one product per block projects them.
        """
        config, positions = self.sensor
        bins = self.shape[1]
        flat = target.reshape(-1)
        for start in range(0, self.size, chunk):
            rows = slice(start, min(start + chunk, self.size))
            basis = self.block_basis(rows)
            if real:
                block = positions[rows.start // bins : rows.stop // bins]
                a = surfel.design(config, block, params, self.fresnel_n, real=True)
                y = torch.view_as_real(flat[rows]).reshape(len(block), 2 * bins).t().reshape(-1)
                if basis is not None:
                    a, y = basis.reduce_major(a), basis.reduce_major(y)
            else:
                a, y = self.design(params, rows), flat[rows]
                if basis is not None:
                    a, y = basis.reduce(a), basis.reduce(y)
            yield a, y

    # -- dictionary rows ---------------------------------------------------------------------------

    def _rows_by_aperture(self, rows):
        """(positions of the distinct apertures of rows, each row's aperture index, its bin)."""
        bins = self.shape[1]
        apertures, which = torch.unique(torch.div(rows, bins, rounding_mode="floor"), return_inverse=True)
        return self.scan.scan_positions_m[apertures], which, torch.remainder(rows, bins)

    def design(self, params, rows):
        """Complex dictionary rows [rows, S]; a slice must cover whole apertures."""
        config, positions = self.sensor
        bins = self.shape[1]
        if isinstance(rows, slice):
            block = positions[rows.start // bins : -(-rows.stop // bins)]
            return surfel.design(config, block, params, self.fresnel_n)
        block, which, bin_ids = self._rows_by_aperture(rows)
        full = surfel.design(config, block, params, self.fresnel_n)
        return full.reshape(len(block), bins, -1)[which, bin_ids]

    def jacobian(self, params, rows, atoms, keys):
        """Column derivatives [rows, atoms, D] for the given parameter keys and row ids."""
        block, which, bin_ids = self._rows_by_aperture(rows)
        subset = {key: value[atoms] for key, value in params.items()}
        derivatives = surfel.jacobian(self.scan.fmcw_config, block, subset, self.fresnel_n)
        return {key: derivatives[key][which, bin_ids] for key in keys}

    # -- model products (CUDA kernels) -------------------------------------------------------------

    def render(self, params, coefficients):
        return surfel.render(*self.sensor, params, coefficients, self.fresnel_n)

    def jvp(self, params, coefficients, tangent, delta_coefficients):
        return surfel.jvp(*self.sensor, params, coefficients, tangent, delta_coefficients, self.fresnel_n)

    def vjp(self, params, coefficients, upstream):
        return surfel.vjp(*self.sensor, params, coefficients, upstream, self.fresnel_n)

    def correlate(self, params, residual, active=None):
        return surfel.correlate(*self.sensor, params, residual.reshape(self.shape), self.fresnel_n, active)

    def correlate_gradient(self, params, residual, include_normals=False):
        return surfel.correlate_gradient(*self.sensor, params, residual.reshape(self.shape), self.fresnel_n,
                                         include_normals)  # fmt: skip

    def correlate_orientations(self, params, residual, bank, table=None):
        return surfel.correlate_orientations(*self.sensor, params, bank, residual.reshape(self.shape),
                                             self.fresnel_n, table)  # fmt: skip

    def orient_best(self, params, residual, bank, energy, real_mode, table=None):
        return surfel.orient_best(*self.sensor, params, bank, residual.reshape(self.shape), energy, real_mode,
                                  self.fresnel_n, table)  # fmt: skip

    # -- spatial-search helpers --------------------------------------------------------------------

    @torch.no_grad()
    def range_gate(self, points, measurement, relative_power, margin_cells, min_fraction):
        """Points whose range falls inside a measured range interval at enough apertures.

        32 evenly spaced apertures with signal threshold their profile against its own
        peak, every interval above the threshold is dilated by margin_cells range
        resolutions, and a point must hit an interval at min_fraction of them
        (dsg_range_gate).
        """
        config, positions = self.sensor
        ids = torch.linspace(0, len(measurement) - 1, min(32, len(measurement)), device=points.device).long()
        power = measurement[ids].abs().square()
        peak = power.amax(-1)
        seen = peak > peak.max() * 1e-6
        power, peak = power[seen], peak[seen]
        spacing = config.range_bin_spacing_m
        reach = math.ceil(margin_cells * config.range_resolution_m / spacing)
        hot = (power >= relative_power * peak[:, None]).float().unsqueeze(1)
        intervals = F.max_pool1d(hot, 2 * reach + 1, stride=1, padding=reach).squeeze(1).int()
        return search.range_gate(points, positions[ids][seen], intervals, spacing, min_fraction)

    @torch.no_grad()
    def range_table(self, residual, oversample=8):
        """Oversampled FFT range correlations of the residual for proposal scores.

        The profiles go back to their ADC samples (inverse FFT), then forward again into
        n_fft * oversample points: the correlation with a unit echo at every off-grid
        range. norm is the matching |kernel|^2 over the observed bins.
        """
        config = self.scan.fmcw_config
        n, samples = config.n_fft, config.adc_samples
        fine = n * oversample
        profiles = residual.reshape(self.shape)
        adc = torch.fft.ifft(profiles, n=n, dim=-1)[..., :samples] * (n / samples)
        correlation = torch.fft.fft(adc, n=fine, dim=-1)
        window = torch.fft.fft(profiles.real.new_ones(samples), n=fine) / samples
        observed = profiles.real.new_zeros(fine)
        observed[: config.num_range_bins * oversample : oversample] = 1
        norm = torch.fft.ifft(torch.fft.fft(observed) * torch.fft.fft(window.abs().square())).real
        return RangeTable(torch.view_as_real(correlation).contiguous(), norm.contiguous(), oversample)


# --- Initializer: range migration ------------------------------------------------------------


def _raster_frame(positions, nu, nv):
    """Origin, pitches and the orthonormal frame (u, v, u x v) of a row-major planar raster."""
    grid = positions.reshape(nu, nv, 3)
    step_u = (grid[-1, 0] - grid[0, 0]) / (nu - 1)
    step_v = (grid[0, -1] - grid[0, 0]) / (nv - 1)
    du, dv = float(step_u.norm()), float(step_v.norm())
    eu, ev = step_u / du, step_v / dv
    return grid[nu // 2, nv // 2], du, dv, torch.stack([eu, ev, torch.linalg.cross(eu, ev)], -1)


def _chirp_samples(scan, dtype):
    """ADC samples [A, S] back from the positive range bins (residual video phase undone)."""
    cfg = scan.fmcw_config
    data = scan.data
    beat = torch.arange(cfg.num_range_bins, device=data.device, dtype=dtype) * (cfg.sample_rate_hz / cfg.n_fft)
    unphased = data * torch.exp(1j * math.pi * beat.square() / cfg.slope_hz_s)
    return torch.fft.ifft(unphased, n=cfg.n_fft, dim=-1)[..., : cfg.adc_samples] * cfg.adc_samples


def _depth_planes(z, wavenumber, depth_samples):
    """Depths at which the field is focused: the points' own planes when they are few and
    regularly spaced, else an even grid with four samples per Nyquist interval of the
    band |kz - K / 2| <= K_max / 2."""
    planes = torch.unique(z)
    if len(planes) < 3:
        regular = True
    else:
        gaps = planes.diff()
        regular = torch.allclose(gaps, gaps.mean().expand(len(gaps)), atol=1e-7, rtol=1e-4)
    if len(planes) <= depth_samples and regular:
        return planes
    z_low, z_high = float(z.min()), float(z.max())
    count = max(depth_samples, 1 + math.ceil((z_high - z_low) * float(wavenumber.max()) * 2 / math.pi))
    return torch.linspace(z_low, z_high, count, device=z.device, dtype=z.dtype)


@torch.no_grad()
def migration(scan, points, aperture_shape, *, depth_samples=96, padding=2, frequency_chunk=16):
    """Relative complex focusing strength of a planar raster scan at world-space points.

    Reference: dsplat/fmcw.py:361-454. The scan must be a complete row-major planar raster
    and the points lie on one side of it. Positive range bins go back to chirp samples, the
    aperture field of every ADC sample is propagated by the angular spectrum (K = 4 pi f / c,
    every propagating replica of an undersampled aperture kept) and the focused volume is
    interpolated at the points. A scalar Green model without obliquity or Fresnel factors:
    an initializer, not a calibrated reflectivity. The frequency sum for every (depth, kx,
    ky) is one CUDA kernel (dsg_migration_focus); frequency_chunk is accepted for the
    reference's signature and has no effect.
    """
    from .kernels import _lib

    del frequency_chunk
    nu, nv = aperture_shape
    cfg = scan.fmcw_config
    device, dtype = points.device, points.dtype
    origin, du, dv, frame = _raster_frame(scan.scan_positions_m, nu, nv)
    local = (points - origin) @ frame
    local[:, 2] = local[:, 2].abs()
    z = local[:, 2]
    flat = float(z.max() - z.min()) < 1e-6
    # zero-padded aperture field per ADC sample, centred, and its 2-D spectrum
    pu, pv = nu * padding, nv * padding
    adc = _chirp_samples(scan, dtype)
    field_ = adc.new_zeros((cfg.adc_samples, pu, pv))
    su, sv = pu // 2 - nu // 2, pv // 2 - nv // 2
    field_[:, su : su + nu, sv : sv + nv] = adc.reshape(nu, nv, -1).permute(2, 0, 1)
    spectrum = torch.fft.fftshift(torch.fft.fft2(torch.fft.ifftshift(field_, dim=(-2, -1))), dim=(-2, -1))
    spectrum = spectrum.to(torch.complex64)
    times = cfg.adc_start_time_s + torch.arange(cfg.adc_samples, device=device, dtype=dtype) / cfg.sample_rate_hz
    wavenumber = (4 * math.pi / cfg.c0_m_s) * (cfg.fc_hz + cfg.slope_hz_s * times)
    k_max = float(wavenumber.max())
    carrier = wavenumber.max() / 2
    depths = _depth_planes(z, wavenumber, 1 if flat else depth_samples)
    # the sampled spectrum is periodic: keep every propagating replica
    copies = (max(1, math.ceil(k_max * du / math.pi)), max(1, math.ceil(k_max * dv / math.pi)))
    qu, qv = pu * copies[0], pv * copies[1]
    dx, dy = du / copies[0], dv / copies[1]
    kx = 2 * math.pi * torch.fft.fftshift(torch.fft.fftfreq(qu, d=dx, device=device, dtype=dtype))
    ky = 2 * math.pi * torch.fft.fftshift(torch.fft.fftfreq(qv, d=dy, device=device, dtype=dtype))
    focused = torch.empty((len(depths), qu, qv, 2), dtype=torch.float32, device=device)
    # every buffer the kernel reads stays referenced here until the launch is queued
    inputs = [torch.view_as_real(spectrum.contiguous()).contiguous(), wavenumber.float().contiguous(),
              kx.float().contiguous(), ky.float().contiguous(), depths.float().contiguous()]  # fmt: skip
    field_spectrum, k32, kx32, ky32, depth32 = inputs
    _lib.call("dsg_migration_focus", _lib.ptr(field_spectrum), cfg.adc_samples, pu, pv, _lib.ptr(k32), _lib.ptr(kx32),
              _lib.ptr(ky32), qu, qv, _lib.ptr(depth32), len(depths), _lib.ptr(focused), _lib.stream(device))  # fmt: skip
    # crop the points' footprint (two cells of margin) from each focused plane
    pitch = local.new_tensor([dx, dy])
    first = torch.floor(local[:, :2].amin(0) / pitch).long() - 2
    last = torch.ceil(local[:, :2].amax(0) / pitch).long() + 2
    (x0, y0), (x1, y1) = first.tolist(), last.tolist()
    planes = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(torch.view_as_complex(focused), dim=(-2, -1))),
                                dim=(-2, -1))  # fmt: skip
    crop = planes[:, x0 + qu // 2 : x1 + qu // 2 + 1, y0 + qv // 2 : y1 + qv // 2 + 1]
    # interpolate with the carrier removed (a centred band), then put it back
    volume = crop * torch.exp(1j * carrier * depths)[:, None, None] * (copies[0] * copies[1] / cfg.adc_samples)
    xy = 2 * (local[:, :2] - first * pitch) / ((last - first) * pitch) - 1
    zz = 2 * (z - z.min()) / (z.max() - z.min()) - 1 if len(depths) > 1 else torch.zeros_like(z)
    where = torch.stack([xy[:, 1], xy[:, 0], zz], -1).reshape(1, 1, 1, -1, 3)
    channels = torch.view_as_real(volume).permute(3, 0, 1, 2).unsqueeze(0)
    sampled = F.grid_sample(channels, where, mode="bilinear", align_corners=True).reshape(2, -1)
    return torch.complex(sampled[0], sampled[1]) * torch.exp(-1j * carrier * z)
