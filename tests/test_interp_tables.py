"""The interpolated correlation form's fixed tables, checked on the CPU.

dsg_surfel_interp_tables returns, without a GPU, the per-chirp tables the interpolated
correlations read (csrc/interp.cu): H (residual -> grid values of Z0 and Z1) and the grid
values of N0 and N1. Here the device arithmetic is restated in float64 NumPy — the grid
values u = r H, the pair's position k0 2^g / P on each grid, the exponential-of-semicircle
weights of the 8 nearest cells and the phase exp(-i pi k0 / P) — and the statistics
interpolated from the library's float32 tables must agree with the oracle's exact sums over
the kept bins (oracle.kernel.dirichlet):

  Z0 = sum_k conj(D(k - k0)) r_k,   Z1 = sum_k conj(D'(k - k0)) r_k,
  N0 = sum_k |D(k - k0)|^2,         N1 = sum_k Re(conj(D) D').
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle.kernel import dirichlet

TAPS = 8
BETA = 2.30 * TAPS


def _tables(samples, pad):
    from dsplat.kernels import _lib

    bins = samples * pad // 2
    correlation = np.zeros(bins * 2 * samples * 4, dtype=np.float32)
    norm = np.zeros(4 * samples * 2, dtype=np.float32)
    status = _lib.library().dsg_surfel_interp_tables(
        samples, pad, correlation.ctypes.data_as(ctypes.c_void_p), correlation.size,
        norm.ctypes.data_as(ctypes.c_void_p), norm.size)  # fmt: skip
    assert status == 0
    h = correlation.astype(np.float64).view(np.complex128).reshape(bins, 2 * samples, 2)
    v = norm.astype(np.float64).reshape(4 * samples, 2)
    return h, v


def _weights(x):
    """Kernel weights of the 8 cells floor(x) - 3 .. floor(x) + 4 at positions x [n]."""
    base = np.floor(x).astype(np.int64)
    taps = base[:, None] + np.arange(-3, 5)[None, :]
    z = 2.0 * (x[:, None] - taps) / TAPS
    a = 1.0 - z * z
    weights = np.where(a > 0, np.exp(BETA * (np.sqrt(np.clip(a, 0, None)) - 1.0)), 0.0)
    return taps, weights


def _interpolated(h, v, residual, k0, samples, pad):
    cells, cells0 = 2 * samples, 4 * samples
    u = residual @ h.reshape(h.shape[0], -1)  # [2 samples * 2] per aperture
    u = u.reshape(cells, 2)
    taps, w = _weights(k0 * 2 / pad)
    phase = np.exp(-1j * np.pi * k0 / pad)
    z0 = phase * (w * u[taps % cells, 0]).sum(1)
    z1 = phase * (w * u[taps % cells, 1]).sum(1)
    taps, w = _weights(k0 * 4 / pad)
    n0 = (w * v[taps % cells0, 0]).sum(1)
    n1 = (w * v[taps % cells0, 1]).sum(1)
    return z0, z1, n0, n1


def _exact(residual, k0, samples, pad):
    bins = samples * pad // 2
    delta = torch.arange(bins, dtype=torch.float64)[None, :] - torch.as_tensor(k0)[:, None]
    d, dp = dirichlet(delta, samples, samples * pad)
    r = torch.as_tensor(residual)[None, :]
    z0 = (d.conj() * r).sum(1)
    z1 = (dp.conj() * r).sum(1)
    n0 = d.abs().square().sum(1)
    n1 = (d.conj() * dp).real.sum(1)
    return z0.numpy(), z1.numpy(), n0.numpy(), n1.numpy()


@pytest.mark.parametrize("samples,pad", [(128, 2), (64, 1), (32, 4), (256, 1)])
def test_interpolated_statistics_match_the_exact_bin_sums(samples, pad):
    h, v = _tables(samples, pad)
    bins = samples * pad // 2
    rng = np.random.default_rng(samples + pad)
    residual = rng.standard_normal(bins) + 1j * rng.standard_normal(bins)
    # positions everywhere on the period, bin centres and half bins included
    k0 = np.concatenate((rng.uniform(0, samples * pad, 3000), np.arange(0, bins, 0.5)))
    got = _interpolated(h, v, residual, k0, samples, pad)
    want = _exact(residual, k0, samples, pad)
    for name, a, b in zip(("Z0", "Z1", "N0", "N1"), got, want, strict=True):
        error = np.abs(a - b).max() / np.abs(b).max()
        assert error < 2e-6, (name, error)


def test_tables_reject_unsupported_chirps():
    from dsplat.kernels import _lib

    buffer = np.zeros(16, dtype=np.float32)
    pointer = buffer.ctypes.data_as(ctypes.c_void_p)
    lib = _lib.library()
    assert lib.dsg_surfel_interp_tables(96, 2, pointer, 16, pointer, 16) != 0  # not a power of two
    assert lib.dsg_surfel_interp_tables(128, 3, pointer, 16, pointer, 16) != 0  # pad
    assert lib.dsg_surfel_interp_tables(128, 2, pointer, 16, pointer, 16) != 0  # buffers too small
