"""FMCW surfel kernels on the GPU against the float64 oracle (parity tests).

Tolerances: the forward (render, design) must be within relative L2 1e-5 of the
float64 closed form; derivatives within 1e-4 relative L2 of the oracle's autograd;
correlations 1e-5 relative to their largest magnitude.
"""

from __future__ import annotations

import pytest
import torch
from conftest import aperture_grid, close, rel_l2, surfels

from oracle import adjoint as oadjoint
from oracle import fmcw as ofmcw

pytestmark = pytest.mark.gpu

FORWARD_TOL = 1e-5
DERIV_TOL = 1e-4


def _cfg(**kw):
    from dsplat import FMCWConfig

    return FMCWConfig(**kw)


def _weights(count, seed=1):
    generator = torch.Generator().manual_seed(seed)
    w = torch.complex(torch.randn(count, generator=generator), torch.randn(count, generator=generator))
    return (w * 1e-2).cuda()


def test_small_forward_workload_is_within_1e_5_of_the_float64_closed_form():
    from dsplat.kernels import surfel as kernel
    from dsplat.workloads import forward_scene

    positions, params, weights = forward_scene()
    config = _cfg()
    out = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    expected = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                            weights.cpu())  # fmt: skip
    assert out.shape == (1024, 128) and out.dtype == torch.complex64
    assert rel_l2(out, expected) < FORWARD_TOL


@pytest.mark.parametrize("pad,fresnel,side", [(2, 0.0, 8), (4, 0.0, 6), (2, 1.6, 8), (1, 0.0, 5)])
def test_render_matches_the_oracle(pad, fresnel, side):
    from dsplat.kernels import surfel as kernel

    config = _cfg(pad_factor=pad) if pad != 1 else _cfg(pad_factor=1, adc_samples=256)
    positions = aperture_grid(side)
    params = surfels(7, seed=pad)
    w = _weights(7)
    out = kernel.render(config, positions, params["centers"], params["normals"], w, fresnel)
    expected = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                            w.cpu(), fresnel)  # fmt: skip
    assert rel_l2(out, expected) < FORWARD_TOL


def test_render_matches_independent_adc_synthesis():
    from dsplat import surfel

    config = _cfg(pad_factor=4)
    positions = aperture_grid(6)
    params = surfels(4)
    reflectivity = torch.rand(4, device="cuda") + 0.5
    rendered = surfel.render(config, positions, params, reflectivity)
    amplitudes = (reflectivity * params["areas"].sqrt()).cpu()
    synthesized = ofmcw.synthesize(positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                                   amplitudes, config)  # fmt: skip
    assert rel_l2(rendered, synthesized) < FORWARD_TOL


def test_empty_and_ragged_inputs():
    from dsplat.kernels import surfel as kernel

    config = _cfg()
    positions = aperture_grid(3)  # 9 apertures: not a multiple of the 16-aperture tile
    params = surfels(33)  # one past a 32-surfel batch
    w = _weights(33)
    out = kernel.render(config, positions, params["centers"], params["normals"], w, 0.0)
    expected = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), w.cpu())
    assert rel_l2(out, expected) < FORWARD_TOL
    none = kernel.render(config, positions, params["centers"][:0], params["normals"][:0], w[:0], 0.0)
    assert none.shape == (9, 128) and bool((none == 0).all())
    # Back-facing surfels render nothing.
    flipped = kernel.render(config, positions, params["centers"], -params["normals"], w, 0.0)
    assert bool((flipped == 0).all())


def test_render_is_deterministic():
    from dsplat.kernels import surfel as kernel
    from dsplat.workloads import forward_scene

    positions, params, weights = forward_scene()
    config = _cfg()
    a = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    b = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    assert torch.equal(a, b)


@pytest.mark.parametrize("real", [True, False])
def test_design_matches_the_oracle(real):
    from dsplat.kernels import surfel as kernel

    config = _cfg()
    positions = aperture_grid(5)
    params = surfels(6)
    out = kernel.design(config, positions, params["centers"], params["normals"], params["areas"], 0.0, real)
    expected = ofmcw.design(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                            params["areas"].cpu(), 0.0, real)  # fmt: skip
    assert out.shape == expected.shape
    assert rel_l2(out, expected) < FORWARD_TOL


def test_jacobian_matches_forward_mode_derivatives_of_the_oracle():
    from dsplat.kernels import surfel as kernel

    config = _cfg()
    positions = aperture_grid(4)
    params = surfels(5)
    cols, dc, dn = kernel.jacobian(config, positions, params["centers"], params["normals"], 0.0)
    pos, cen, nrm = positions.cpu().double(), params["centers"].cpu().double(), params["normals"].cpu().double()
    assert rel_l2(cols, ofmcw.columns(pos, cen, nrm, config)) < FORWARD_TOL
    for key, got in (("centers", dc), ("normals", dn)):
        for axis in range(3):
            tangent_c = torch.zeros_like(cen)
            tangent_n = torch.zeros_like(nrm)
            (tangent_c if key == "centers" else tangent_n)[:, axis] = 1.0
            _, expected = torch.func.jvp(lambda c, n: ofmcw.columns(pos, c, n, config), (cen, nrm),
                                         (tangent_c, tangent_n))  # fmt: skip
            assert rel_l2(got[..., axis], expected) < DERIV_TOL


def test_jvp_and_vjp_match_the_oracle_and_are_adjoint(fmcw):
    model, params, b = fmcw
    config, positions = model.sensor
    generator = torch.Generator().manual_seed(7)
    b = (b.to(torch.complex64) * torch.exp(1j * torch.arange(5, device="cuda")))
    tangent = {
        "centers": (torch.randn(5, 3, generator=generator) * 1e-4).cuda(),
        "normals": (torch.randn(5, 3, generator=generator) * 1e-2).cuda(),
        "areas": (torch.randn(5, generator=generator) * 1e-6).cuda(),
    }
    db = torch.complex(torch.randn(5, generator=generator), torch.randn(5, generator=generator)).cuda()
    jvp = model.jvp(params, b, tangent, db)
    root = params["areas"].sqrt()
    w, dw = b * root, db * root + b * tangent["areas"] / (2 * root)
    expected = ofmcw.jvp(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), w.cpu(),
                         tangent["centers"].cpu(), tangent["normals"].cpu(), dw.cpu())  # fmt: skip
    assert rel_l2(jvp, expected) < DERIV_TOL
    upstream = torch.complex(torch.randn(model.shape, generator=generator),
                             torch.randn(model.shape, generator=generator)).cuda()  # fmt: skip
    grads, gb = model.vjp(params, b, upstream)
    gc, gn, gw = ofmcw.vjp(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                           w.cpu(), upstream.cpu())  # fmt: skip
    assert rel_l2(grads["centers"], gc) < DERIV_TOL
    assert rel_l2(grads["normals"], gn) < DERIV_TOL
    assert rel_l2(gb, gw * root.cpu()) < DERIV_TOL
    left = (upstream.conj() * jvp).real.sum().double()
    right = sum((grads[k].double() * v.double()).sum() for k, v in tangent.items())
    right = right + (gb.conj() * db).real.sum().double()
    torch.testing.assert_close(left, right, rtol=1e-4, atol=1e-12)
    leaves = {k: v.clone().requires_grad_() for k, v in params.items()}
    b_leaf = b.clone().requires_grad_()
    (upstream.conj() * model.render(leaves, b_leaf)).real.sum().backward()
    for key in params:
        close(leaves[key].grad, grads[key], 1e-5)
    close(b_leaf.grad, gb, 1e-5)


@pytest.mark.parametrize("pad", [2, 4])
def test_vjp_near_the_peak_and_across_pads(pad):
    """Surfels whose peaks sit on, near and between bins exercise the nearest-bin path."""
    from dsplat.kernels import surfel as kernel

    config = _cfg(pad_factor=pad)
    positions = aperture_grid(4)
    params = surfels(9, seed=3)
    spacing = config.range_bin_spacing_m
    # Put surfel 0 exactly on a bin for aperture 0 and surfel 1 a hair off it.
    p0 = positions[0].cpu().double()
    for s, frac in ((0, 0.0), (1, 1e-4), (2, 0.5)):
        c = params["centers"][s].cpu().double()
        r = (p0 - c).norm()
        target = (torch.round(r / spacing) + frac) * spacing
        params["centers"][s] = (p0 + (c - p0) * target / r).float().cuda()
    w = _weights(9)
    generator = torch.Generator().manual_seed(4)
    upstream = torch.complex(torch.randn(16, config.num_range_bins, generator=generator),
                             torch.randn(16, config.num_range_bins, generator=generator)).cuda()  # fmt: skip
    gc, gn, gw = kernel.vjp(config, positions, params["centers"], params["normals"], w, upstream, 0.0)
    ec, en, ew = ofmcw.vjp(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                           w.cpu(), upstream.cpu())  # fmt: skip
    assert rel_l2(gc, ec) < DERIV_TOL and rel_l2(gn, en) < DERIV_TOL and rel_l2(gw, ew) < DERIV_TOL
    # the reference VJP kernel's own formulas (class sums, nearest bin apart) in float64
    ac, an, aw = oadjoint.vjp(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                              w.cpu(), upstream.cpu())  # fmt: skip
    assert rel_l2(gc, ac) < DERIV_TOL and rel_l2(gn, an) < DERIV_TOL and rel_l2(gw, aw) < DERIV_TOL
    dc = torch.randn_like(params["centers"]) * 1e-4
    dn = torch.randn_like(params["normals"]) * 1e-2
    dw = _weights(9, seed=5)
    jv = kernel.jvp(config, positions, params["centers"], params["normals"], w, dc, dn, dw, 0.0)
    ej = ofmcw.jvp(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), w.cpu(),
                   dc.cpu(), dn.cpu(), dw.cpu())  # fmt: skip
    assert rel_l2(jv, ej) < DERIV_TOL
    out = kernel.render(config, positions, params["centers"], params["normals"], w, 0.0)
    eo = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), w.cpu())
    assert rel_l2(out, eo) < FORWARD_TOL


def test_correlations_and_their_gradients_match_the_oracle(fmcw):
    from dsplat.kernels import surfel as kernel

    model, params, _ = fmcw
    config, positions = model.sensor
    residual = model.scan.data
    candidates = surfels(40, seed=11)
    cen, nrm = candidates["centers"], candidates["normals"]
    corr, norm = kernel.correlate(config, positions, cen, nrm, residual, 0.0)
    ec, en = ofmcw.correlate(config, positions.cpu(), cen.cpu(), nrm.cpu(), residual.cpu())
    close(corr, ec, 1e-5)
    close(norm, en, 1e-5)
    for include in (False, True):
        c, n, dc, dn = kernel.correlate_gradient(config, positions, cen, nrm, residual, 0.0, include)
        xc, xn, xdc, xdn = ofmcw.correlate_gradient(config, positions.cpu(), cen.cpu(), nrm.cpu(),
                                                    residual.cpu(), include_normals=include)  # fmt: skip
        close(c, xc, 1e-5)
        close(n, xn, 1e-5)
        assert rel_l2(dc, xdc) < DERIV_TOL
        assert rel_l2(dn, xdn) < DERIV_TOL


def test_normal_bank_scores_match_the_oracle(fmcw):
    from dsplat.certificate import fibonacci_sphere
    from dsplat.kernels import surfel as kernel

    model, params, _ = fmcw
    config, positions = model.sensor
    residual = model.scan.data
    candidates = surfels(50, seed=12)
    bank = fibonacci_sphere(24, "cuda")
    corr, norm = kernel.correlate_orientations(config, positions, candidates["centers"],
                                               candidates["normals"], bank, residual, 0.0)  # fmt: skip
    ec, en = ofmcw.correlate_orientations(config, positions.cpu(), candidates["centers"].cpu(),
                                          candidates["normals"].cpu(), bank.cpu(), residual.cpu())  # fmt: skip
    close(corr, ec, 1e-5)
    close(norm, en, 1e-5)
    table = model.range_table(residual, 8)
    tc, tn = kernel.correlate_orientations(config, positions, candidates["centers"],
                                           candidates["normals"], bank, residual, 0.0, table)  # fmt: skip
    oc, on = ofmcw.correlate_orientations(
        config, positions.cpu(), candidates["centers"].cpu(), candidates["normals"].cpu(), bank.cpu(),
        residual.cpu(), table=(table.correlation.cpu(), table.norm.cpu(), 8))  # fmt: skip
    close(tc, oc, 1e-4)
    close(tn, on, 1e-4)
    close(tc, ec, 3e-2)  # the FFT table approximates the exact scores (reference bound)
    close(tn, en, 3e-2)


def test_normal_bank_scores_ragged_sizes_and_fresnel():
    """49 apertures (a partial aperture chunk), 41 bank normals (two normal chunks), 37
    candidates (a partial block) and a Fresnel factor, exact and table paths."""
    from dsplat import FMCWConfig, FMCWModel, Scan
    from dsplat.certificate import fibonacci_sphere
    from dsplat.kernels import surfel as kernel

    config = FMCWConfig()
    positions = aperture_grid(7)
    truth = surfels(4, seed=21)
    weights = torch.tensor([1.0, -0.5, 0.7, 0.3], device="cuda").to(torch.complex64)
    empty = Scan(torch.zeros((len(positions), config.num_range_bins), dtype=torch.complex64, device="cuda"),
                 positions, config)  # fmt: skip
    residual = FMCWModel(empty, fresnel_n=1.5).render(truth, weights)
    model = FMCWModel(Scan(residual, positions, config), fresnel_n=1.5)
    candidates = surfels(37, seed=22)
    bank = fibonacci_sphere(40, "cuda")
    corr, norm = kernel.correlate_orientations(config, positions, candidates["centers"], candidates["normals"],
                                               bank, residual, 1.5)  # fmt: skip
    ec, en = ofmcw.correlate_orientations(config, positions.cpu(), candidates["centers"].cpu(),
                                          candidates["normals"].cpu(), bank.cpu(), residual.cpu(), 1.5)  # fmt: skip
    assert corr.shape == (37, 41) and norm.shape == (37, 41)
    close(corr, ec, 1e-5)
    close(norm, en, 1e-5)
    table = model.range_table(residual, 8)
    tc, tn = kernel.correlate_orientations(config, positions, candidates["centers"], candidates["normals"],
                                           bank, residual, 1.5, table)  # fmt: skip
    oc, on = ofmcw.correlate_orientations(
        config, positions.cpu(), candidates["centers"].cpu(), candidates["normals"].cpu(), bank.cpu(),
        residual.cpu(), 1.5, table=(table.correlation.cpu(), table.norm.cpu(), 8))  # fmt: skip
    close(tc, oc, 1e-4)
    close(tn, on, 1e-4)


def test_correlate_active_set_matches_the_full_launch(fmcw):
    """dsg_surfel_correlate_active: candidates s with s mod period < count equal the full
    correlate; the rest are zero. Three blocks of 70 candidates, 23 active per block."""
    from dsplat.kernels import surfel as kernel

    model, _, _ = fmcw
    config, positions = model.sensor
    residual = model.scan.data
    cand = surfels(210, seed=31)
    corr, norm = kernel.correlate(config, positions, cand["centers"], cand["normals"], residual, 0.0)
    count = torch.tensor([23], dtype=torch.int32, device="cuda")
    ac, an = kernel.correlate(config, positions, cand["centers"], cand["normals"], residual, 0.0,
                              active=(count, 70))  # fmt: skip
    live = torch.arange(210, device="cuda") % 70 < 23
    assert torch.equal(ac[live], corr[live]) and torch.equal(an[live], norm[live])
    assert float(ac[~live].abs().max()) == 0.0 and float(an[~live].abs().max()) == 0.0


@pytest.mark.parametrize("pad,samples,fresnel", [(2, 128, 0.0), (1, 256, 1.6), (4, 100, 0.0)])
def test_synthesize_matches_the_float64_oracle(pad, samples, fresnel):
    """groundtruth.synthesize (dsg_synthesize_adc + torch.fft) against the float64 ADC
    synthesis of the oracle: the same scan up to complex64 storage (rel-L2 1e-6). 300
    surfels cover a partial 256-surfel chunk; 100 samples a partial 16-sample block."""
    from dsplat.groundtruth import synthesize

    config = _cfg(pad_factor=pad, adc_samples=samples)
    positions = aperture_grid(6)
    params = surfels(300, seed=41)
    generator = torch.Generator().manual_seed(42)
    amplitudes = torch.complex(torch.rand(300, generator=generator) + 0.5,
                               torch.randn(300, generator=generator) * 0.3).cuda() * 0.01  # fmt: skip
    scan = synthesize(positions, params["centers"], params["normals"], amplitudes, config, fresnel)
    expected = ofmcw.synthesize(positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), amplitudes.cpu(),
                                config, fresnel)  # fmt: skip
    assert scan.data.dtype == torch.complex64 and scan.data.shape == expected.shape
    assert rel_l2(scan.data, expected) < 1e-6


@pytest.mark.parametrize("samples,pad,side,count", [(128, 2, 32, 256), (64, 4, 9, 37), (256, 1, 8, 70), (16, 4, 5, 9)])
def test_forward_through_adc_samples_matches_the_oracle(samples, pad, side, count):
    """dsg_surfel_render_samples + the n_fft-point FFT against the float64 closed form and the
    bin-sum forward, with ragged surfel counts (the last chunk by plain loads), several
    segments and a misaligned weight view (no bulk copies)."""
    from dsplat.kernels import surfel as kernel

    config = _cfg(adc_samples=samples, pad_factor=pad)
    positions = aperture_grid(side)
    params = surfels(count, seed=samples + pad, spread=0.03)
    w = _weights(count, seed=pad)
    expected = ofmcw.render(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(), w.cpu())
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    y = kernel.render_samples(config, positions, params["centers"], params["normals"], w, 0.0, status=status)
    via_samples = torch.fft.fft(y, n=config.n_fft, dim=1)[:, : config.num_range_bins]
    bins = kernel.render(config, positions, params["centers"], params["normals"], w, 0.0)
    assert int(status.item()) == 0
    assert rel_l2(via_samples, expected) < FORWARD_TOL
    assert rel_l2(via_samples, bins) < FORWARD_TOL
    with kernel.render_form("samples"):
        same = kernel.render(config, positions, params["centers"], params["normals"], w, 0.0)
    torch.testing.assert_close(same, via_samples, rtol=0, atol=0)
    # a weight view that starts 8 bytes into its storage: plain loads, same values
    padded = torch.zeros(count + 1, dtype=torch.complex64, device="cuda")
    padded[1:] = w
    y2 = kernel.render_samples(config, positions, params["centers"], params["normals"], padded[1:], 0.0)
    close(y2, y, 1e-6)


def test_forward_through_adc_samples_at_full_size():
    """The 128^2-array, 2000-surfel sphere cap: every row within 1e-5 of the bin-sum forward
    (itself within 1e-5 of float64 at this size, tests/test_full_size_gpu.py)."""
    from dsplat import FMCWConfig
    from dsplat.kernels import surfel as kernel
    from dsplat.workloads import sphere_cap

    config = FMCWConfig()
    positions, params, reflectivity = sphere_cap(device="cuda")
    weights = (reflectivity * params["areas"].sqrt()).to(torch.complex64)
    bins = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    with kernel.render_form("samples"):
        via_samples = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    assert rel_l2(via_samples, bins) < FORWARD_TOL
