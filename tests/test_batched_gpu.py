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


@pytest.mark.parametrize("mode,with_normals,frozen_z", [("real", True, False), ("complex", True, False),
                                                        ("real", False, True)])  # fmt: skip
def test_fused_ascent_iterations_match_the_pytorch_iterations(fmcw, mode, with_normals, frozen_z):
    """Three iterations of the fused kernels (dsg_trials, dsg_ascent_partition,
    dsg_ascent_select, dsg_ascent_update) against the PyTorch iteration on the same state:
    the same accepted steps, centers within a thousandth of their step scale, normals within
    1e-5, values, gradients and BFGS inverses within 1e-4."""
    from dsplat import ParameterConfig
    from dsplat.ascent import _closures, _fused_iteration, _iteration
    from dsplat.certificate import CertificateSearchConfig, _controls

    model, params, _ = fmcw
    residual = model.scan.data
    generator = torch.Generator().manual_seed(4)
    start = {k: v.repeat(6, *([1] * (v.ndim - 1))).contiguous() for k, v in params.items()}
    start["centers"] = (start["centers"] + (3e-4 * torch.randn(start["centers"].shape, generator=generator)).cuda())
    base = fmcw_specs()
    center_spec = base["centers"]
    if frozen_z:
        center_spec = ParameterConfig(trainable=(True, True, False), scale=0.0005, lower=(-0.02, -0.02, 0.28),
                                      upper=(0.02, 0.02, 0.32))  # fmt: skip
    specs = {"centers": center_spec}
    if with_normals:
        specs["normals"] = base["normals"]
    masks = {key: spec.mask(start[key]) for key, spec in specs.items()}
    controls = _controls(start["centers"], center_spec, specs.get("normals"), masks)
    config = CertificateSearchConfig(peaks=30, separation=0, iterations=3)
    fractions = [0.5**b for b in range(config.backtracks)]
    ascent, score = _closures(model, residual, masks, specs, mode)
    value, grad = score(start, True)
    grad = ascent(start, grad)
    count, dim = grad.shape
    eye = torch.eye(dim, device="cuda").expand(count, dim, dim)
    reference = (dict(start), value, grad, eye.clone())
    state = ({k: v.clone() for k, v in start.items()}, value.clone(), grad.clone(), eye.contiguous().clone())
    iterate = _iteration(model, residual, controls, masks, specs, config, mode, fractions, eye)
    power = residual.abs().square().sum().double().clamp(min=1e-30).reshape(1)
    fused = _fused_iteration(model, residual, power, controls, specs, config, mode, fractions)
    stuck = torch.zeros(count, dtype=torch.uint8, device="cuda")
    for _ in range(config.iterations):
        reference = iterate(*reference)
        fused(*state, stuck)
        moved = (state[0]["centers"] != start["centers"]).any(1)
        expected_moved = (reference[0]["centers"] != start["centers"]).any(1)
        assert torch.equal(moved, expected_moved)
        close(state[0]["centers"], reference[0]["centers"], 2e-6)
        close(state[0]["normals"], reference[0]["normals"], 1e-5)
        close(state[1], reference[1], 1e-4)
        close(state[2], reference[2], 1e-4)
        close(state[3], reference[3], 1e-4)
    if frozen_z:
        assert torch.equal(state[0]["centers"][:, 2], start["centers"][:, 2])
    # every candidate flagged stuck is one the PyTorch iterations did not move in the last round
    assert bool(((stuck == 0) | ~(state[0]["centers"] != reference[0]["centers"]).any(1)).all())


@pytest.mark.parametrize("count", [1, 1000, 3000])
def test_ascent_partition_is_the_stable_pending_first_order(count):
    """dsg_ascent_partition over several 1024-candidate chunks: the slots are the inverse
    of the stable argsort of the improvement flags, the pending count and the batch rows
    follow them, and the selection takes the first improving fraction."""
    from dsplat.kernels import search

    generator = torch.Generator().manual_seed(count)
    fractions = 4
    corr = torch.complex(torch.randn(count, generator=generator), torch.randn(count, generator=generator)).cuda()
    norm = torch.rand(count, generator=generator).cuda() + 0.5
    areas = torch.rand(count, generator=generator).cuda() + 0.5
    value = torch.rand(count, generator=generator).cuda()
    power = torch.tensor([1.7], dtype=torch.float64, device="cuda")
    trial_centers = torch.randn(fractions, count, 3, generator=generator).cuda()
    trial_normals = torch.randn(fractions, count, 3, generator=generator).cuda()
    improved, position, pending, batch_centers, batch_normals = search.ascent_partition(
        corr, norm, areas, power, True, value, trial_centers, trial_normals)  # fmt: skip
    c = (corr * areas.sqrt()).to(torch.complex128)
    certificate = (c.real.square() / (norm * areas).double() / 1.7).float()
    expected = certificate > value
    assert torch.equal(improved.bool(), expected)
    order = torch.argsort(expected.to(torch.int8), stable=True)
    assert torch.equal(position.long(), torch.argsort(order))
    assert int(pending) == int((~expected).sum())
    rows = batch_centers.reshape(fractions - 1, count, 3)
    assert torch.equal(rows, trial_centers[1:, order])
    assert torch.equal(batch_normals.reshape(fractions - 1, count, 3), trial_normals[1:, order])
    # second phase: raw correlations of the batch rows, area applied by slot owner
    corr2 = torch.complex(torch.randn((fractions - 1) * count, generator=generator),
                          torch.zeros((fractions - 1) * count)).cuda()  # fmt: skip
    norm2 = torch.ones((fractions - 1) * count, device="cuda")
    centers, normals = torch.zeros(count, 3, device="cuda"), torch.zeros(count, 3, device="cuda")
    new_centers, new_normals, accepted = search.ascent_select(
        corr2, norm2, areas, power, True, value, improved, position, trial_centers, trial_normals, centers,
        normals, True)  # fmt: skip
    owner_root, owner_area = areas.sqrt()[order].repeat(fractions - 1), areas[order].repeat(fractions - 1)
    scaled = (corr2.real * owner_root).double()
    later = (scaled.square() / (norm2 * owner_area).double() / 1.7).float().reshape(fractions - 1, count)
    better = later > value[order][None]
    slot_pending = torch.arange(count, device="cuda") < int(pending)
    better &= slot_pending[None]
    for i in range(0, count, max(1, count // 97)):
        if expected[i]:
            assert bool(accepted[i]) and torch.equal(new_centers[i], trial_centers[0, i])
            continue
        p = int(position[i])
        hits = better[:, p].nonzero().flatten()
        if len(hits):
            r = int(hits[0]) + 1
            assert bool(accepted[i]) and torch.equal(new_centers[i], trial_centers[r, i])
            assert torch.equal(new_normals[i], trial_normals[r, i])
        else:
            assert not bool(accepted[i]) and torch.equal(new_centers[i], centers[i])


@pytest.mark.parametrize("n", [1, 37, 64, 65, 128, 130, 150, 513, 1000, 2256])
@pytest.mark.parametrize("complex_mode", [False, True])
def test_triangular_inverse_across_the_recursion(n, complex_mode):
    """dsg_triangular_inverse at sizes on both sides of the 64-row diagonal blocks and
    through several levels of trmm halving (130 and 150 split 128 + 2 and 128 + 22, where a
    lower level's product is the largest): L^-1 to 1e-11 (well conditioned factor), zero
    above the diagonal."""
    from dsplat.kernels import search

    dtype = torch.complex128 if complex_mode else torch.float64
    generator = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(2 * n + 3, n, dtype=dtype, device="cuda", generator=generator)
    factor = torch.linalg.cholesky(x.mH @ x / len(x) + 0.1 * torch.eye(n, dtype=dtype, device="cuda"))
    inverse = search.triangular_inverse(factor)
    expected = torch.linalg.inv(factor)
    assert float((inverse - expected).norm() / expected.norm()) < 1e-11
    assert float(inverse.triu(1).abs().max()) == 0.0 if n > 1 else True


def test_triangular_inverse_reports_the_first_zero_pivot():
    """A zero on the diagonal at row 70 (second 64-row block) gives status 71."""
    from dsplat.kernels import _lib, search
    from dsplat.kernels._lib import call, ptr

    n = 200
    factor = torch.eye(n, dtype=torch.float64, device="cuda") * 2
    factor[70, 70] = 0.0
    factor[150, 150] = 0.0
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    nbytes = _lib.query("dsg_triangular_inverse_workspace_bytes", n, 0)
    work, nbytes = _lib.workspace(nbytes, factor.device)
    call("dsg_triangular_inverse", ptr(factor), n, 0, ptr(work), nbytes, ptr(info), _lib.stream(factor.device))
    assert int(info) == 71
    healthy = search.triangular_inverse(torch.eye(n, dtype=torch.float64, device="cuda") * 2)
    assert torch.equal(healthy, torch.eye(n, dtype=torch.float64, device="cuda") * 0.5)
