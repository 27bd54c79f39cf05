"""The two forms of the aperture-reduced kernels on the GPU: interpolated and exact.

dsg_surfel_correlate, _correlate_active, _correlate_gradient and _vjp evaluate per pair
the statistics Z0, Z1, N0, N1 of the closed-form kernel over the kept bins either by
summing every bin (DSG_CORRELATION_EXACT) or by interpolating them from per-aperture
tables (DSG_CORRELATION_INTERP, the default; a type-2 nonuniform FFT accurate to about
1e-7). Both must match the float64 oracle at the kernels' tolerances (correlations 1e-5 of
the largest magnitude, derivatives 1e-4 relative L2) and each other within 2e-5 of the
largest magnitude, including chirps with pad 1 and 4, peaks beyond the kept bins,
back-facing pairs and ragged sizes.
"""

from __future__ import annotations

import pytest
import torch
from conftest import aperture_grid, close, rel_l2, surfels

from oracle import fmcw as ofmcw

pytestmark = pytest.mark.gpu

DERIV_TOL = 1e-4
FORMS_AGREE = 2e-5  # of the largest magnitude: the float32 rounding of the derivative sums


def _upstream(apertures, bins, seed):
    generator = torch.Generator().manual_seed(seed)
    return torch.complex(torch.randn(apertures, bins, generator=generator),
                         torch.randn(apertures, bins, generator=generator)).cuda()  # fmt: skip


def _weights(count, seed):
    generator = torch.Generator().manual_seed(seed)
    return torch.complex(torch.randn(count, generator=generator), torch.randn(count, generator=generator)).cuda()


def _both(fn):
    from dsplat.kernels import surfel as kernel

    out = {}
    for form in ("interp", "exact"):
        with kernel.correlation_form(form):
            out[form] = fn()
    return out


@pytest.mark.parametrize("samples,pad", [(128, 2), (64, 1), (32, 4)])
def test_both_forms_match_the_oracle(samples, pad):
    from dsplat import FMCWConfig
    from dsplat.kernels import surfel as kernel

    config = FMCWConfig(adc_samples=samples, pad_factor=pad)
    positions = aperture_grid(7)  # 49 apertures: ragged chunks
    cand = surfels(37, seed=samples + pad, spread=0.05)  # peaks spread over many bins
    cen, nrm = cand["centers"], cand["normals"]
    residual = _upstream(len(positions), config.num_range_bins, seed=3)
    weights = _weights(len(cen), seed=4)
    pc, cc, nc = positions.cpu(), cen.cpu(), nrm.cpu()
    ec, en = ofmcw.correlate(config, pc, cc, nc, residual.cpu())
    gc, gn, gw = ofmcw.vjp(config, pc, cc, nc, weights.cpu(), residual.cpu())
    xc, xn, xdc, xdn = ofmcw.correlate_gradient(config, pc, cc, nc, residual.cpu(), include_normals=True)
    got = _both(lambda: (kernel.correlate(config, positions, cen, nrm, residual, 0.0),
                         kernel.vjp(config, positions, cen, nrm, weights, residual, 0.0),
                         kernel.correlate_gradient(config, positions, cen, nrm, residual, 0.0, True)))  # fmt: skip
    for form, ((corr, norm), (vc, vn, vw), (c, n, dc, dn)) in got.items():
        close(corr, ec, 1e-5)
        close(norm, en, 1e-5)
        assert rel_l2(vc, gc) < DERIV_TOL, form
        assert rel_l2(vn, gn) < DERIV_TOL, form
        assert rel_l2(vw, gw) < DERIV_TOL, form
        close(c, xc, 1e-5)
        close(n, xn, 1e-5)
        assert rel_l2(dc, xdc) < DERIV_TOL, form
        assert rel_l2(dn, xdn) < DERIV_TOL, form
    for a, b in zip(got["interp"], got["exact"], strict=True):
        for x, y in zip(a, b, strict=True):
            close(x, y, FORMS_AGREE)


def test_forms_agree_at_the_ascent_size_with_back_facing_pairs_and_far_peaks():
    """2048 apertures x 1100 candidates (three partial 32-surfel blocks); some candidates
    face away from every aperture and some lie beyond the kept range bins."""
    from dsplat import FMCWConfig
    from dsplat.kernels import surfel as kernel
    from dsplat.workloads import sphere_cap

    config = FMCWConfig()
    positions, params, _ = sphere_cap(side=128, surfel_count=1100, device="cuda")
    positions = positions[::8].contiguous()
    cen, nrm = params["centers"].clone(), params["normals"].clone()
    nrm[::50] = -nrm[::50]  # back-facing
    cen[7::97, 2] += 1.5  # peaks past the last kept bin
    residual = _upstream(len(positions), config.num_range_bins, seed=9)
    weights = _weights(len(cen), seed=10)
    active = torch.tensor([200], dtype=torch.int32, device="cuda")
    got = _both(lambda: (kernel.correlate(config, positions, cen, nrm, residual, 0.0),
                         kernel.correlate_gradient(config, positions, cen, nrm, residual, 0.0, False),
                         kernel.vjp(config, positions, cen, nrm, weights, residual, 0.0),
                         kernel.correlate(config, positions, cen, nrm, residual, 0.0, active=(active, 550))))  # fmt: skip
    for a, b in zip(got["interp"], got["exact"], strict=True):
        for x, y in zip(a, b, strict=True):
            close(x, y, FORMS_AGREE)
    corr, _ = got["interp"][3]
    inactive = (torch.arange(len(cen), device="cuda") % 550) >= 200
    assert bool((corr[inactive] == 0).all())


@pytest.mark.parametrize("samples,pad", [(128, 2), (64, 4)])
def test_tabled_calls_equal_the_residual_calls_bitwise(samples, pad):
    """A residual's interpolation tables computed once (dsg_surfel_residual_tables) give
    the correlations, the active-set correlations and the gradients bit for bit."""
    from dsplat import FMCWConfig
    from dsplat.kernels import surfel as kernel

    config = FMCWConfig(adc_samples=samples, pad_factor=pad)
    positions = aperture_grid(9)  # 81 apertures
    cand = surfels(77, seed=5, spread=0.04)
    cen, nrm = cand["centers"], cand["normals"]
    residual = _upstream(len(positions), config.num_range_bins, seed=12)
    active = torch.tensor([20], dtype=torch.int32, device="cuda")
    with kernel.correlation_form("interp"):
        tables = kernel.residual_tables(config, residual)
        plain = (kernel.correlate(config, positions, cen, nrm, residual, 0.0),
                 kernel.correlate(config, positions, cen, nrm, residual, 0.0, active=(active, 40)),
                 kernel.correlate_gradient(config, positions, cen, nrm, residual, 0.0, True),
                 kernel.correlate_gradient(config, positions, cen, nrm, residual, 0.0, False))  # fmt: skip
        tabled = (kernel.correlate(config, positions, cen, nrm, None, 0.0, tables=tables),
                  kernel.correlate(config, positions, cen, nrm, None, 0.0, active=(active, 40), tables=tables),
                  kernel.correlate_gradient(config, positions, cen, nrm, None, 0.0, True, tables=tables),
                  kernel.correlate_gradient(config, positions, cen, nrm, None, 0.0, False, tables=tables))  # fmt: skip
        short = kernel.residual_tables(config, residual, derivative=False)
        corr_short = kernel.correlate(config, positions, cen, nrm, None, 0.0, tables=short)
    for a, b in zip(plain, tabled, strict=True):
        for x, y in zip(a, b, strict=True):
            assert torch.equal(x, y)
    assert torch.equal(corr_short[0], plain[0][0]) and torch.equal(corr_short[1], plain[0][1])
