"""Host-side solver logic that needs no GPU: parameter constraints, the pooled-fit
elimination, regularized inverses and utilities (CPU float64)."""

from __future__ import annotations

import math

import pytest
import torch


def test_unit_vectors_with_a_frozen_component_stay_unit():
    from dsplat import ParameterConfig

    spec = ParameterConfig(trainable=(True, True, False), normalize=True)
    reference = torch.nn.functional.normalize(torch.tensor([[0.3, 0.4, -0.6]]), dim=1)
    value = spec.project(torch.tensor([[2.0, -1.0, 5.0]]), reference)
    assert value[0, 2] == reference[0, 2]
    torch.testing.assert_close(value.norm(dim=1), torch.ones(1))


def test_unit_vector_tangent_matches_the_projection_with_a_frozen_component():
    from dsplat import ParameterConfig

    spec = ParameterConfig(trainable=(True, False, True), normalize=True)
    generator = torch.Generator().manual_seed(3)
    value = torch.nn.functional.normalize(torch.randn(4, 3, generator=generator, dtype=torch.float64), dim=1)
    for axis in (0, 2):
        step = torch.zeros_like(value)
        step[:, axis] = 1e-6
        numeric = (spec.project(value + step, value) - spec.project(value - step, value)) / 2e-6
        torch.testing.assert_close(spec.tangent(step / 1e-6, value), numeric, atol=1e-7, rtol=0)


def test_a_free_part_of_zero_length_takes_the_reference_direction():
    from dsplat import ParameterConfig

    spec = ParameterConfig(trainable=(True, False, True), normalize=True)
    reference = torch.tensor([[0.6, 0.8, 0.0]])
    torch.testing.assert_close(spec.project(torch.tensor([[0.0, 0.8, 0.0]]), reference), reference)


def test_unit_vector_with_no_free_radius_has_zero_derivatives():
    from dsplat import ParameterConfig

    spec = ParameterConfig(trainable=(True, False, True), normalize=True)
    value = torch.tensor([[0.0, 1.0, 0.0]], dtype=torch.float64)
    direction = torch.tensor([[1.0, 0.0, 2.0]], dtype=torch.float64)
    numeric = (spec.project(value + 1e-6 * direction, value) - spec.project(value - 1e-6 * direction, value)) / 2e-6
    torch.testing.assert_close(numeric, torch.zeros_like(value))
    torch.testing.assert_close(spec.tangent(direction, value), numeric)
    jacobian = torch.eye(3, dtype=value.dtype).reshape(3, 1, 3)
    torch.testing.assert_close(spec.differential(jacobian, value), torch.zeros(3, 1, 2, dtype=value.dtype))


@pytest.mark.parametrize("trainable", [True, (True, False, True)])
def test_normalizing_without_any_reference_direction_raises(trainable):
    from dsplat import ParameterConfig

    spec = ParameterConfig(trainable=trainable, normalize=True)
    value = torch.zeros(1, 3)
    with pytest.raises(ValueError, match="reference direction"):
        spec.project(value, value)


def test_periodic_bounds_and_frozen_components():
    from dsplat import ParameterConfig
    from dsplat.parameters import periodic_delta

    spec = ParameterConfig(trainable=(True, False), period=(24, 20), lower=None)
    value = spec.project(torch.tensor([[25.5, 3.0]]), torch.tensor([[1.0, 7.0]]))
    torch.testing.assert_close(value, torch.tensor([[1.5, 7.0]]))
    torch.testing.assert_close(periodic_delta(torch.tensor([[23.0, -11.0]]), (24, 20)),
                               torch.tensor([[-1.0, 9.0]]))  # fmt: skip
    boxed = ParameterConfig(lower=(0.0, 0.0, 0.3), upper=(0.1, 0.1, 0.4))
    torch.testing.assert_close(boxed.project(torch.tensor([[-1.0, 0.05, 9.0]]), torch.zeros(1, 3)),
                               torch.tensor([[0.0, 0.05, 0.4]]))  # fmt: skip


def test_backward_elimination_follows_brute_force_refits():
    from dsplat.replacement import backward_elimination

    generator = torch.Generator().manual_seed(4)
    x = torch.randn(20, 8, generator=generator, dtype=torch.float64)
    h, q = x.T @ x, x.T @ torch.randn(20, generator=generator, dtype=torch.float64)

    def objective(keep):
        keep = list(keep)
        return float(-q[keep] @ torch.linalg.solve(h[keep][:, keep], q[keep]))

    alive, expected = set(range(8)), []
    for _ in range(3):
        best = min(alive, key=lambda j: objective(alive - {j}))
        expected.append(best)
        alive.remove(best)
    assert backward_elimination(torch.linalg.inv(h), q, 3).tolist() == expected


def test_limited_elimination_removes_at_most_limit_marked_unknowns():
    from dsplat.replacement import backward_elimination

    generator = torch.Generator().manual_seed(6)
    x = torch.randn(30, 10, generator=generator, dtype=torch.float64)
    h, q = x.T @ x, x.T @ torch.randn(30, generator=generator, dtype=torch.float64)
    limited = torch.arange(10) < 6
    removed = backward_elimination(torch.linalg.inv(h), q, 5, limited, 2)
    assert int(limited[removed].sum()) <= 2 and len(set(removed.tolist())) == 5


def test_regularized_inverse_shifts_by_a_fraction_of_the_largest_eigenvalue():
    from dsplat.replacement import regularized_inverse

    h = torch.diag(torch.tensor([0.0, 1.0, 2.0, 3.0, 4.0, 10.0], dtype=torch.float64))
    inverse = regularized_inverse(h, 1e-3)
    shifted = h + 0.01 * torch.eye(6, dtype=torch.float64)
    torch.testing.assert_close(inverse, torch.linalg.inv(shifted), rtol=0, atol=1e-6 * 100)


@pytest.mark.parametrize("seed", [1, 3, 4, 28])
def test_regularized_inverse_has_a_positive_scalar_shift_and_scales_with_the_gram(seed):
    from dsplat.replacement import regularized_inverse

    generator = torch.Generator().manual_seed(seed)
    x = torch.randn(30, 6, dtype=torch.float64, generator=generator)
    h = x.T @ x
    inverse = regularized_inverse(h, 1e-3)
    difference = torch.linalg.inv(inverse) - h
    shift = difference.diag().mean()
    assert 0 < shift <= 1e-3 * torch.linalg.eigvalsh(h)[-1] * (1 + 1e-10)
    torch.testing.assert_close(difference, shift * torch.eye(6, dtype=h.dtype), atol=1e-12, rtol=1e-9)
    torch.testing.assert_close(regularized_inverse(7 * h, 1e-3) * 7, inverse)


def test_utility_marks_a_duplicated_column_redundant():
    from dsplat.replacement import utility

    x = torch.randn(40, 4, dtype=torch.float64, generator=torch.Generator().manual_seed(2))
    x = torch.cat((x, x[:, :1]), 1)
    efficiency = 2 * utility(x.T @ x, torch.zeros(5, dtype=torch.float64))
    assert efficiency[0] < 1e-6 and efficiency[4] < 1e-6 and (efficiency[1:4] > 0.1).all()


def test_solve_of_a_singular_system_predicts_like_the_pseudoinverse():
    from dsplat.varpro import solve

    generator = torch.Generator().manual_seed(8)
    basis = torch.randn(6, 3, dtype=torch.float64, generator=generator)
    h = basis @ basis.T
    q = basis @ torch.randn(3, dtype=torch.float64, generator=generator)
    x = solve(h, q)
    torch.testing.assert_close(basis.T @ x, basis.T @ (torch.linalg.pinv(h, hermitian=True) @ q),
                               rtol=0, atol=1e-8 * float(q.abs().max()))  # fmt: skip
    torch.testing.assert_close(h @ x, q, rtol=0, atol=1e-8 * float(q.abs().max()))
    assert torch.equal(solve(torch.zeros(3, 3, dtype=torch.float64), torch.zeros(3, dtype=torch.float64)),
                       torch.zeros(3, dtype=torch.float64))  # fmt: skip


def test_pcg_solves_a_symmetric_positive_system():
    from dsplat.varpro import pcg

    generator = torch.Generator().manual_seed(9)
    m = torch.randn(12, 12, dtype=torch.float64, generator=generator)
    h = m @ m.T + torch.eye(12, dtype=torch.float64)
    b = torch.randn(12, dtype=torch.float64, generator=generator)
    x = pcg(lambda v: h @ v, b, h.diag(), iterations=200, tolerance=1e-12)
    torch.testing.assert_close(x, torch.linalg.solve(h, b), rtol=1e-8, atol=1e-10)


def test_candidate_grid_and_fibonacci_bank():
    from dsplat.certificate import candidate_grid, fibonacci_sphere

    grid = candidate_grid([0.0, -1.0], [1.0, 1.0], 0.3, device="cpu")
    assert grid.shape == (5 * 8, 2) and grid.min(0).values.tolist() == [0, -1]
    bank = fibonacci_sphere(24, "cpu")
    torch.testing.assert_close(bank.norm(dim=1), torch.ones(24))
    assert abs(float(bank[:, 2].mean())) < 1e-6


def test_row_basis_rank_of_the_sphere_cap_band():
    """The shared basis of the 128^2 / 2000-surfel box has rank 30 (float64 SVD on the CPU)."""
    from dsplat import FMCWConfig

    from oracle import fmcw as ofmcw

    config = FMCWConfig()
    low, high = 62.0, 90.8
    count = max(2 * config.adc_samples, int(16 * (high - low)) + 1)
    response = ofmcw.range_response(config, low, high, count)
    values = torch.linalg.svdvals(response)
    rank = int((values > torch.finfo(torch.float32).eps / 128 * values[0]).sum())
    assert 25 <= rank <= 35


@pytest.mark.parametrize("complex_mode", [False, True])
def test_refined_solve_reaches_float64_accuracy_or_declines(complex_mode):
    """Float32 factor + float64 refinement: float64-accurate on a system of condition ~1e4,
    and None (the float64 path takes over) on one of condition ~1e10."""
    from dsplat.varpro import refined_solve

    generator = torch.Generator().manual_seed(3)
    dtype = torch.complex128 if complex_mode else torch.float64
    q, _ = torch.linalg.qr(torch.randn(80, 80, generator=generator, dtype=dtype))
    rhs = torch.randn(80, generator=generator, dtype=dtype)
    for condition, expect in ((1e4, True), (1e10, False)):
        values = torch.logspace(0, -math.log10(condition), 80, dtype=torch.float64)
        h = (q * values.to(dtype)) @ q.mH
        x = refined_solve(h, rhs)
        if expect:
            exact = torch.linalg.solve(h, rhs)
            assert float((x - exact).norm() / exact.norm()) < 1e-10
        else:
            assert x is None


def test_shifted_refined_solve_matches_the_float64_shift():
    """A float32 Gram of rank n/2 fails float32 Cholesky; its shifted system solved from a
    float32 factor with float64 refinement equals the float64 factorization's solution."""
    from dsplat.varpro import shifted_cholesky, shifted_refined_solve

    generator = torch.Generator().manual_seed(5)
    n = 200
    a = torch.randn(3 * n, n // 2, generator=generator) @ torch.randn(n // 2, n, generator=generator) / n
    h = a.T @ a / len(a)
    assert int(torch.linalg.cholesky_ex(h)[1]) != 0
    q = torch.randn(n, 1, generator=generator)
    floor = n * torch.finfo(torch.float32).eps
    expected = torch.cholesky_solve(q.double(), shifted_cholesky(h, floor))
    x = shifted_refined_solve(h, q, floor)
    assert x is not None and float((x - expected).norm() / expected.norm()) < 1e-10


def test_ascent_spec_packs_the_parameter_configs():
    """DsgAscentSpec of the certificate ascent: width, unit-vector flags, scales and the
    free-component masks of centers (one frozen axis) and normals."""
    from dsplat import ParameterConfig
    from dsplat.kernels.search import ascent_spec

    specs = {"centers": ParameterConfig(trainable=(True, False, True), scale=5e-4),
             "normals": ParameterConfig(scale=0.1, normalize=True)}  # fmt: skip
    spec = ascent_spec(specs)
    assert spec.width == 6
    assert list(spec.normalize) == [0, 1]
    assert list(spec.scale) == pytest.approx([5e-4, 0.1])
    assert list(spec.mask) == [1.0, 0.0, 1.0, 1.0, 1.0, 1.0]
    centers_only = ascent_spec({"centers": ParameterConfig(scale=2.0)})
    assert centers_only.width == 3 and list(centers_only.mask)[:3] == [1.0, 1.0, 1.0]


def test_fused_ascent_takes_only_surfel_candidates():
    """The fused ascent needs a surfel model on CUDA whose candidates hold centers, normals
    and areas, and at most 16 backtracking fractions; anything else keeps the PyTorch loop."""
    from types import SimpleNamespace

    from dsplat.ascent import _fusable

    class Tensorish:
        is_cuda = True

    model = SimpleNamespace(scan=None, sensor=None, fresnel_n=0.0)
    surfel = {"centers": Tensorish(), "normals": Tensorish(), "areas": Tensorish()}
    assert _fusable(model, surfel, [1.0, 0.5])
    assert not _fusable(model, dict(surfel, reflectivity=Tensorish()), [1.0])
    assert not _fusable(model, surfel, [0.5**b for b in range(17)])
    assert not _fusable(SimpleNamespace(sensor=None, fresnel_n=0.0), surfel, [1.0])
    host = dict(surfel, centers=SimpleNamespace(is_cuda=False))
    assert not _fusable(model, host, [1.0])
