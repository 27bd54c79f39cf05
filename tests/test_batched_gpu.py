"""The batched execution (DSFWConfig.batched) against the sequential reference structure."""

from __future__ import annotations

import itertools

import pytest
import torch
from conftest import close, fmcw_specs, surfels

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("separation,period", [(0.0, None), (0.05, None), (1.5, (24.0, 20.0))])
def test_device_distinct_equals_the_sequential_selection(separation, period):
    from dsplat.kernels import search
    from dsplat.replacement import _distinct

    generator = torch.Generator().manual_seed(7)
    dim = 3 if period is None else 2
    scale = 1.0 if period is None else 24.0
    points = (torch.rand(3000, dim, generator=generator) * scale).cuda()
    points[10] = points[3]  # an exact duplicate must collide even at separation 0
    occupied = (torch.rand(200, dim, generator=generator) * scale).cuda()
    occupied[5] = points[20]
    scores = torch.rand(3000, generator=generator).cuda()
    scores[::17] = -torch.inf
    scores[40] = scores[41]
    for width in (1, 64, 1000):
        got = search.distinct(scores, points, occupied, period, separation, width)
        expected = _distinct(scores, points, occupied, period, separation, width)
        assert got.tolist() == expected.tolist()


@pytest.mark.parametrize("complex_mode", [False, True])
def test_device_elimination_equals_the_eager_loop(complex_mode):
    """dsg_backward_elimination against the PyTorch loop: the same removal order, with and
    without a limit on the marked unknowns, for a real and a Hermitian inverse."""
    from dsplat.replacement import backward_elimination

    generator = torch.Generator().manual_seed(5)
    dtype = torch.complex128 if complex_mode else torch.float64
    x = torch.randn(300, 60, generator=generator, dtype=dtype)
    h = x.mH @ x
    q = x.mH @ torch.randn(300, generator=generator, dtype=dtype)
    inverse, q = torch.linalg.inv(h).cuda(), q.cuda()
    limited = torch.arange(60, device="cuda") < 40
    for lim, l in ((None, 0), (limited, 5)):
        eager = backward_elimination(inverse, q, 20, lim, l)
        for _ in range(2):
            device = backward_elimination(inverse, q, 20, lim, l, on_device=True)
            assert torch.equal(eager, device)


def test_batched_certificate_search_matches_the_sequential_search(fmcw):
    from dsplat.certificate import CertificateSearchConfig, search_certificate

    model, params, coefficients = fmcw
    residual = model.scan.data
    generator = torch.Generator().manual_seed(2)
    start = {k: v.repeat(6, *([1] * (v.ndim - 1))) for k, v in params.items()}
    start["centers"] = start["centers"] + (3e-4 * torch.randn(start["centers"].shape, generator=generator)).cuda()
    specs = fmcw_specs()
    config = CertificateSearchConfig(peaks=30, separation=0, iterations=12)
    seq, seq_scores = search_certificate(model, residual, start, specs["centers"], config, "real",
                                         normal_spec=specs["normals"])  # fmt: skip
    bat, bat_scores = search_certificate(model, residual, start, specs["centers"], config, "real",
                                         normal_spec=specs["normals"], batched=True)  # fmt: skip
    close(bat_scores, seq_scores, 1e-4)
    close(bat["centers"], seq["centers"], 1e-4)
    # A second search of the same shapes replays the cached graph with new inputs: a
    # different residual and start, against a fresh sequential search.
    residual2 = residual * 0.7 + 0.3 * residual.flip(0)
    start2 = dict(start, centers=start["centers"] + (2e-4 * torch.randn(start["centers"].shape,
                                                                          generator=generator)).cuda())  # fmt: skip
    seq2, seq2_scores = search_certificate(model, residual2, start2, specs["centers"], config, "real",
                                           normal_spec=specs["normals"])  # fmt: skip
    bat2, bat2_scores = search_certificate(model, residual2, start2, specs["centers"], config, "real",
                                           normal_spec=specs["normals"], batched=True)  # fmt: skip
    close(bat2_scores, seq2_scores, 1e-4)
    close(bat2["centers"], seq2["centers"], 1e-4)


def test_batched_steps_never_raise_the_objective(fmcw):
    from dsplat import DSFWConfig, initialize, step

    model, params, _ = fmcw
    config = DSFWConfig(batch=5, lm_gain_ratio=0, joint_apertures=16, screen_apertures=16,
                        batched=True, gram="bf16x3")  # fmt: skip
    state = initialize(model, model.scan.data, surfels(5, seed=9), config, candidates=params,
                       parameters=fmcw_specs())  # fmt: skip
    for _ in range(4):
        state = step(state, config)
    objectives = [entry["objective"] for entry in state.history]
    assert all(b <= a for a, b in itertools.pairwise(objectives)) and objectives[-1] < objectives[0]


@pytest.mark.parametrize("complex_mode", [False, True])
def test_factor_form_elimination_equals_the_eager_loop(complex_mode):
    """The batched replacement eliminates from X = L^-1 (trtri) instead of the inverse
    X^H X (potri): the triangular inverse matches torch's and the removal order matches the
    PyTorch loop on the full inverse, with and without a limit."""
    from dsplat.kernels import search
    from dsplat.replacement import backward_elimination, regularized_inverse, regularized_inverse_factor

    generator = torch.Generator().manual_seed(7)
    dtype = torch.complex128 if complex_mode else torch.float64
    x = torch.randn(400, 90, generator=generator, dtype=dtype)
    h = (x.mH @ x).cuda()
    q = (x.mH @ torch.randn(400, generator=generator, dtype=dtype)).cuda()
    floor = len(h) * torch.finfo(torch.float32).eps
    factor = torch.linalg.cholesky(h)
    inverse_factor = search.triangular_inverse(factor)
    assert torch.allclose(inverse_factor, torch.linalg.inv(factor), rtol=1e-9, atol=1e-12)
    inverse = regularized_inverse(h, floor)
    xfac = regularized_inverse_factor(h, floor)
    assert torch.allclose(xfac.mH @ xfac, inverse, rtol=1e-8, atol=1e-10 * float(inverse.abs().max()))
    limited = torch.arange(90, device="cuda") < 50
    for lim, lmt in ((None, 0), (limited, 7)):
        eager = backward_elimination(inverse, q, 30, lim, lmt)
        device = backward_elimination(xfac, q, 30, lim, lmt, on_device=True, factored=True)
        assert torch.equal(eager, device)


def test_factor_form_elimination_at_the_pooled_size():
    """2256 unknowns (2000 support + 256 pooled), complex and real: the column of the
    inverse factor staged in shared memory is 36 KB (complex), above the default 48 KB
    once the static arrays are added."""
    from dsplat.kernels import search
    from dsplat.replacement import backward_elimination

    for dtype in (torch.float64, torch.complex128):
        generator = torch.Generator().manual_seed(11)
        x = torch.randn(2600, 2256, generator=generator, dtype=dtype).cuda()
        h = x.mH @ x
        q = x.mH @ torch.randn(2600, generator=generator, dtype=dtype).cuda()
        factor = search.triangular_inverse(torch.linalg.cholesky(h))
        inverse = factor.mH @ factor
        eager = backward_elimination(inverse, q, 12)
        device = backward_elimination(factor, q, 12, on_device=True, factored=True)
        assert torch.equal(eager, device)
