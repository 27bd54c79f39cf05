"""Dirichlet atoms on a spectral grid: the signal-level measurement model.

An atom is a center [D] in bin units (one to three axes) with a complex amplitude, its
coefficient. Its spectrum at every grid bin is the product over axes of the windowed
Dirichlet kernel of that axis, evaluated by the CUDA spectral kernels
(dsplat.kernels.spectral). Behaviour of the reference's dsplat/spectral.py:16-120; the
grid's bin coordinates are built once per device and reused by every product.
"""

from __future__ import annotations

from dataclasses import dataclass
from math import prod

import torch

from .kernels import spectral as kernel

_BIN_TABLES: dict = {}


@dataclass(frozen=True)
class SpectralGrid:
    shape: tuple[int, ...]  # FFT length per axis, one to three axes
    samples: tuple[int, ...] | None = None  # observed samples per axis; None: the FFT length
    window: str = "rect"  # rect, hann, hamming or kaiser
    beta: float = 14.0  # Kaiser shape
    radius: float = 0.0  # kernel support in bins; zero keeps the exact, untruncated response

    def __post_init__(self):
        if self.samples is None:
            object.__setattr__(self, "samples", self.shape)

    @property
    def size(self):
        return prod(self.shape)

    def bins(self, device="cuda"):
        """Coordinates [size, D] (float32) of every grid bin, in row-major order."""
        key = (tuple(self.shape), torch.device(device))
        table = _BIN_TABLES.get(key)
        if table is None:
            axes = [torch.arange(n, device=device, dtype=torch.float32) for n in self.shape]
            table = torch.cartesian_prod(*axes).reshape(-1, len(self.shape))
            _BIN_TABLES[key] = table
        return table.clone()


@dataclass(frozen=True)
class SpectralModel:
    """Atoms with centers [S, D] on one grid; it has no apertures."""

    grid: SpectralGrid
    row_alignment = 1
    apertures = 0

    @property
    def shape(self):
        return self.grid.shape

    @property
    def size(self):
        return self.grid.size

    def prepare(self, specs):
        """Nothing to precompute: every bin is observed."""
        return self

    def _bins(self, params):
        return self.grid.bins(params["centers"].device)

    def design(self, params, rows):
        return kernel.design(self.grid, params["centers"], self._bins(params)[rows])

    def jacobian(self, params, rows, atoms, keys):
        derivatives = kernel.design(self.grid, params["centers"][atoms], self._bins(params)[rows], derivatives=True)
        return {"centers": derivatives[1]}

    # The model's products cover the whole grid, so they run in the separable form: per-axis
    # kernel tables (dsg_spectral_axis_tables) combined by complex matrix products.

    def render(self, params, coefficients):
        return kernel.render_on_grid(self.grid, params["centers"], coefficients).reshape(self.shape)

    def jvp(self, params, coefficients, tangent, delta_coefficients):
        change = kernel.jvp_grid(self.grid, params["centers"], coefficients, tangent["centers"], delta_coefficients)
        return change.reshape(self.shape)

    def vjp(self, params, coefficients, upstream):
        centers, weights = kernel.vjp_grid(self.grid, params["centers"], coefficients, upstream)
        return {"centers": centers}, weights

    def correlate(self, params, residual, active=None):
        """a^H r and |a|^2 of every atom (active is ignored: every atom is scored).

        Atoms sitting exactly on every grid bin in order (the candidate set of a full
        search) are correlated as one FFT convolution; any other set streams dictionary
        blocks of at most 2^24 elements.
        """
        centers = params["centers"]
        bins = self._bins(params)
        flat = residual.reshape(-1)
        if centers.shape == bins.shape and torch.equal(centers, bins):
            atom = kernel.design(self.grid, torch.zeros_like(centers[:1]), bins).reshape(self.shape)
            product = torch.fft.fftn(residual.reshape(self.shape)) * torch.fft.fftn(atom).conj()
            energy = atom.abs().square().sum()
            return torch.fft.ifftn(product).reshape(-1), energy.expand(len(centers))
        block = max(1, 2**24 // len(centers))
        corr = flat.new_zeros(len(centers))
        norm = flat.real.new_zeros(len(centers))
        for start in range(0, self.size, block):
            a = self.design(params, slice(start, start + block))
            corr += a.mH @ flat[start : start + block]
            norm += a.abs().square().sum(0)
        return corr, norm

    def blocks(self, params, target, real, chunk):
        """Least-squares blocks of chunk bins; real blocks stack (re, im) rows per bin."""
        flat = target.reshape(-1)
        for start in range(0, self.size, chunk):
            rows = slice(start, start + chunk)
            a, y = self.design(params, rows), flat[rows]
            if real:
                a = torch.view_as_real(a).transpose(1, 2).reshape(-1, a.shape[1])
                y = torch.view_as_real(y).reshape(-1)
            yield a, y

    def sample_rows(self, count, seed, device):
        """Evenly spread rows (deterministic; every row once count reaches the grid size)."""
        return torch.linspace(0, self.size - 1, min(count, self.size), device=device).long()
