"""VarPro, replacement, refinement and search on the GPU against dense linear algebra.

The scenarios and acceptance bounds mirror the reference's own solver and search
tests (tests/test_solver.py, tests/test_search.py, tests/test_fmcw.py of
Asixa/Dirichlet-Splatting), run here through the CUDA kernels.
"""

from __future__ import annotations

import itertools
import math

import pytest
import torch
from conftest import aperture_grid, close, fmcw_specs, surfels

pytestmark = pytest.mark.gpu


def test_streamed_normal_equations_match_dense_products(fmcw):
    from dsplat import DSFWConfig
    from dsplat.varpro import normal_equations

    model, params, _ = fmcw
    model = model.prepare(fmcw_specs())
    y = model.scan.data.flatten()
    a = model.design(params, slice(0, model.size)).to(torch.complex128)
    m = model.size
    for gram_mode in ("fp32", "bf16x3"):
        # Two-aperture blocks give several float64 folds of the float32 Gram.
        config = DSFWConfig(row_chunk=2 * model.shape[1], gram=gram_mode)
        gram, rhs = normal_equations(model, params, model.scan.data, config)
        close(gram, (a.H @ a).real / m, 1e-4)
        close(rhs, (a.H @ y.to(torch.complex128)).real / m, 1e-4)
    gram, rhs = normal_equations(model, params, model.scan.data, DSFWConfig(coefficients="complex"))
    close(gram, a.H @ a / m, 1e-4)
    close(rhs, a.H @ y.to(torch.complex128) / m, 1e-4)


@pytest.mark.parametrize("pad", [2, 4])
def test_row_basis_preserves_the_normal_equations(pad):
    from dsplat import FMCWConfig, FMCWModel, Scan
    from dsplat.fmcw import response_basis

    config = FMCWConfig(pad_factor=pad)
    data = torch.zeros((36, config.num_range_bins), dtype=torch.complex64, device="cuda")
    model = FMCWModel(Scan(data, aperture_grid(6), config))
    a = model.design(surfels(6), slice(0, model.size))
    spacing = config.range_bin_spacing_m
    reduced = response_basis(config, 0.28 / spacing, 0.33 / spacing, "cuda").reduce(a)
    close(reduced.H @ reduced, a.H @ a, 1e-4)


def test_varpro_minimizes_the_ridge_objective(spectral):
    from dsplat import DSFWConfig
    from dsplat.varpro import varpro

    model, params, b = spectral
    target = model.render(params, b)
    trial = {"centers": params["centers"] + 0.3}
    config = DSFWConfig(coefficients="complex", ridge=1e-3)
    coefficients, prediction, loss, _, _ = varpro(model, trial, target, config)
    a = model.design(trial, slice(0, model.size)).to(torch.complex128)
    m = model.size
    h = a.H @ a / m + 1e-3 * torch.eye(3, device="cuda")
    expected = torch.linalg.solve(h, a.H @ target.flatten().to(torch.complex128) / m)
    close(coefficients, expected, 1e-4)
    rendered = (prediction - target).abs().square().mean() + 1e-3 * coefficients.abs().square().sum()
    assert abs(loss - float(rendered)) <= 1e-5 * float(rendered)


def test_one_column_exchange_equals_a_full_refit(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.varpro import exchange_varpro, varpro

    model, params, _ = fmcw
    config = DSFWConfig()
    start = {**params, "centers": params["centers"] + 1e-4}
    state = initialize(model, model.scan.data, start, config, parameters=fmcw_specs())
    proposal = {k: v.clone() for k, v in state.params.items()}
    proposal["centers"][2] = params["centers"][2]
    fast = exchange_varpro(state, proposal, 2, config)
    full = varpro(model, proposal, model.scan.data, config)
    close(fast.coefficients, full.coefficients, 1e-3)
    assert abs(fast.objective - full.objective) <= 1e-3 * full.objective


def test_complex_exchange_equals_a_full_refit(spectral):
    from dsplat import DSFWConfig, initialize
    from dsplat.varpro import exchange_varpro, varpro

    model, params, b = spectral
    target = model.render(params, b)
    config = DSFWConfig(coefficients="complex", ridge=1e-6)
    state = initialize(model, target, {"centers": params["centers"] + 0.2}, config)
    proposal = {"centers": state.params["centers"].clone()}
    proposal["centers"][1] = params["centers"][1]
    fast = exchange_varpro(state, proposal, 1, config)
    full = varpro(model, proposal, target, config)
    close(fast.coefficients, full.coefficients, 1e-3)


def test_merged_replacement_restores_displaced_surfels(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.replacement import merge_support

    model, params, _ = fmcw
    moved = surfels(5, seed=7)
    config = DSFWConfig(batch=5, screen_apertures=0)
    state = initialize(model, model.scan.data, moved, config, candidates=params, parameters=fmcw_specs())
    after, replaced = merge_support(state, config, state.candidates)
    assert replaced > 0 and after.objective < state.objective and len(after.coefficients) == 5


def test_utility_replacement_recovers_a_misplaced_tone(spectral):
    from dsplat import DSFWConfig, ParameterConfig, initialize
    from dsplat.replacement import replace_one

    model, params, b = spectral
    target = model.render(params, b)
    wrong = params["centers"].clone()
    wrong[1] = torch.tensor([20.0, 2.0], device="cuda")
    config = DSFWConfig(coefficients="complex", replacement="utility")
    state = initialize(model, target, {"centers": wrong}, config, candidates={"centers": model.grid.bins()},
                       parameters={"centers": ParameterConfig(period=model.shape)})  # fmt: skip
    after, replaced = replace_one(state, config, state.candidates)
    assert replaced == 1 and after.objective < 0.1 * state.objective


def test_reduced_gradient_is_half_the_derivative_of_the_projected_objective(spectral):
    from dsplat import DSFWConfig, ParameterConfig
    from dsplat.refinement import reduced_system

    model, params, b = spectral
    target = model.render(params, b)
    specs = {"centers": ParameterConfig(scale=0.5)}
    config = DSFWConfig(coefficients="complex", ridge=1e-4)
    rows = torch.arange(model.size, device="cuda")
    trial = {"centers": params["centers"] + torch.tensor([[0.2, -0.1]], device="cuda")}
    _, gradient = reduced_system(model, trial, target, specs, config, rows)

    def projected(centers):
        a = model.design({"centers": centers}, rows).to(torch.complex128)
        y = target.flatten().to(torch.complex128)
        c = torch.linalg.solve(a.H @ a / len(a) + 1e-4 * torch.eye(3, device="cuda"), a.H @ y / len(a))
        return float((a @ c - y).abs().square().mean() + 1e-4 * c.abs().square().sum())

    direction = torch.randn_like(trial["centers"])
    h = 1e-2
    numeric = (projected(trial["centers"] + h * 0.5 * direction)
               - projected(trial["centers"] - h * 0.5 * direction)) / (2 * h)  # fmt: skip
    assert abs(2 * float(gradient @ direction.flatten()) - numeric) <= 2e-2 * abs(numeric)


def test_joint_system_is_symmetric_and_pcg_matches_a_dense_solve(spectral):
    from dsplat import DSFWConfig, ParameterConfig
    from dsplat.refinement import joint_system
    from dsplat.varpro import pcg

    model, params, b = spectral
    target = model.render(params, b)
    trial = {"centers": params["centers"] + 0.1}
    config = DSFWConfig(coefficients="complex", ridge=1e-4)
    matvec, gradient, diagonal, _ = joint_system(model, trial, b, target, {"centers": ParameterConfig()},
                                                 config, 0)  # fmt: skip
    columns = torch.eye(len(gradient), device="cuda")
    dense = torch.stack([matvec(column) for column in columns], 1).double()
    close(dense, dense.T, 1e-4)
    assert torch.linalg.eigvalsh((dense + dense.T) / 2)[0] > 0
    solution = pcg(matvec, -gradient, diagonal, iterations=200, tolerance=1e-7)
    close(solution, torch.linalg.solve(dense, -gradient.double()), 1e-3)


@pytest.mark.parametrize("iterations,tolerance", [(16, 1e-3), (40, 1e-9)])
def test_graph_replayed_pcg_matches_the_eager_loop(fmcw, iterations, tolerance):
    """The batched slide's PCG (first iteration eager, the rest replayed from a captured CUDA
    graph with the stop rule as a device flag) against the eager loop on the same FMCW
    joint system: same iterates up to rounding, also when the stop rule fires early."""
    from dsplat import DSFWConfig
    from dsplat.refinement import joint_system
    from dsplat.varpro import pcg

    model, params, b = fmcw
    trial = {**params, "centers": params["centers"] + 2e-4}
    matvec, gradient, diagonal, _ = joint_system(model, trial, b, model.scan.data, fmcw_specs(), DSFWConfig(), 0)
    eager = pcg(matvec, -gradient, diagonal, iterations=iterations, tolerance=tolerance)
    replayed = pcg(matvec, -gradient, diagonal, iterations=iterations, tolerance=tolerance, capture=True)
    assert bool(torch.isfinite(replayed).all())
    close(replayed, eager, 1e-4)


def test_graph_kept_across_slides_matches_the_eager_loop(fmcw):
    """The batched joint slide's PCG graph, captured once and replayed for a second system
    after its static inputs are refilled (other geometry, coefficients and aperture subset
    of the same shapes), against the eager loop of each system."""
    from dsplat import DSFWConfig
    from dsplat.refinement import _JOINT_GRAPHS, _graphed_joint_pcg, joint_system
    from dsplat.varpro import pcg

    model, params, b = fmcw
    config = DSFWConfig(batched=True)
    _JOINT_GRAPHS.clear()
    for shift, seed, scale in ((2e-4, 0, 1.0), (-3e-4, 5, 1.3)):
        ids, sub = model.sample_apertures(40, seed)
        trial = {**params, "centers": params["centers"] + shift}
        pieces = {}
        matvec, gradient, diagonal, _ = joint_system(sub, trial, b * scale, model.scan.data[ids], fmcw_specs(),
                                                     config, seed, pieces=pieces)  # fmt: skip
        eager = pcg(matvec, -gradient, diagonal, iterations=config.cg_iterations, tolerance=config.cg_tolerance)
        kept = _graphed_joint_pcg(sub, trial, fmcw_specs(), config, pieces, -gradient, diagonal)
        assert bool(torch.isfinite(kept).all())
        close(kept, eager, 1e-4)
    assert len(_JOINT_GRAPHS) == 1  # the second system replayed the first one's graph


def test_fmcw_joint_system_is_symmetric(fmcw):
    from dsplat import DSFWConfig
    from dsplat.refinement import joint_system

    model, params, b = fmcw
    trial = {**params, "centers": params["centers"] + 2e-4}
    matvec, gradient, _, _ = joint_system(model, trial, b, model.scan.data, fmcw_specs(), DSFWConfig(), 0)
    columns = torch.eye(len(gradient), device="cuda")
    dense = torch.stack([matvec(column) for column in columns], 1).double()
    close(dense, dense.T, 1e-3)


def test_screened_steps_never_raise_the_objective(fmcw):
    from dsplat import DSFWConfig, initialize, step

    model, params, _ = fmcw
    config = DSFWConfig(batch=5, lm_gain_ratio=0, joint_apertures=16, screen_apertures=16)
    state = initialize(model, model.scan.data, surfels(5, seed=9), config, candidates=params,
                       parameters=fmcw_specs())  # fmt: skip
    for _ in range(4):
        state = step(state, config)
    objectives = [entry["objective"] for entry in state.history]
    assert all(b <= a for a, b in itertools.pairwise(objectives)) and objectives[-1] < objectives[0]


def test_screened_acceptance_keeps_better_and_rejects_worse_proposals(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.varpro import accept, screen_bar

    model, params, _ = fmcw
    config = DSFWConfig()
    start = {**params, "centers": params["centers"] + 1e-4}
    state = initialize(model, model.scan.data, start, config, parameters=fmcw_specs())
    ids, subset = state.model.sample_apertures(16, 0)
    screen = screen_bar((subset, state.target[ids]), state.params, config)
    worse = {**start, "centers": start["centers"] + 0.005}
    assert accept(state, worse, config, screen) is None
    assert accept(state, params, config, screen).objective < state.objective


def test_unconfigured_parameters_stay_fixed(fmcw):
    from dsplat import DSFWConfig, initialize, step

    model, params, _ = fmcw
    specs = fmcw_specs()
    del specs["areas"]
    config = DSFWConfig(batch=5, lm_gain_ratio=0, screen_apertures=0)
    state = initialize(model, model.scan.data, surfels(5, seed=3), config, candidates=params, parameters=specs)
    assert torch.equal(step(state, config).params["areas"], state.params["areas"])


def test_pooled_statistics_match_a_full_stream(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.replacement import pooled_statistics
    from dsplat.varpro import normal_equations

    model, params, _ = fmcw
    config = DSFWConfig()
    state = initialize(model, model.scan.data, surfels(5, seed=2), config, parameters=fmcw_specs())
    pool = {k: torch.cat((v, params[k])) for k, v in state.params.items()}
    gram, rhs = pooled_statistics(state, pool, config)
    expected_gram, expected_rhs = normal_equations(model, pool, model.scan.data, config)
    close(gram, expected_gram, 1e-4)
    close(rhs, expected_rhs, 1e-4)


def test_streamed_spectral_correlation_matches_the_dictionary(spectral):
    model, params, b = spectral
    residual = model.render(params, b)
    candidates = {"centers": torch.rand(50, 2, device="cuda") * 20}
    corr, norm = model.correlate(candidates, residual)
    a = model.design(candidates, slice(0, model.size))
    close(corr, a.H @ residual.flatten(), 1e-4)
    close(norm, a.abs().square().sum(0), 1e-4)


def test_dense_lm_moves_tones_back(spectral):
    from dsplat import DSFWConfig, ParameterConfig, initialize
    from dsplat.refinement import dense_slide

    model, params, b = spectral
    target = model.render(params, b)
    config = DSFWConfig(coefficients="complex", lm_solver="dense", lm_steps=5, lm_rows=model.size,
                        screen_apertures=0)  # fmt: skip
    specs = {"centers": ParameterConfig(period=model.shape, scale=0.5)}
    state = initialize(model, target, {"centers": params["centers"] + 0.15}, config, parameters=specs)
    after, accepted = dense_slide(state, config)
    assert accepted > 0 and after.objective < 1e-3 * state.objective


def test_dense_lm_on_fmcw_rows_improves_the_fit(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.refinement import dense_slide

    model, params, _ = fmcw
    config = DSFWConfig(lm_solver="dense", lm_steps=3, lm_rows=4096, screen_apertures=0)
    start = {**params, "centers": params["centers"] + 1e-4}
    state = initialize(model, model.scan.data, start, config, parameters=fmcw_specs())
    after, accepted = dense_slide(state, config)
    assert accepted > 0 and after.objective < state.objective


def test_geometry_step_backs_off_while_it_gains_little(spectral):
    from dsplat import DSFWConfig, ParameterConfig, initialize, step

    model, params, b = spectral
    target = model.render(params, b)
    wrong = params["centers"].clone()
    wrong[1] = torch.tensor([20.0, 2.0], device="cuda")
    config = DSFWConfig(coefficients="complex", replacement="utility", lm_solver="dense", lm_rows=model.size,
                        lm_gain_ratio=1e9)  # fmt: skip
    specs = {"centers": ParameterConfig(period=model.shape, scale=0.5)}
    state = initialize(model, target, {"centers": wrong}, config, candidates={"centers": model.grid.bins()},
                       parameters=specs)  # fmt: skip
    state = step(state, config)
    assert state.lm_wait == 1 and state.lm_skip == 1
    state = step(state, config)
    assert state.history[-1]["lm_accepted"] == 0 and state.lm_skip == 0


def test_default_config_runs_on_a_spectral_grid_wider_than_the_aperture_subsets():
    from dsplat import DSFWConfig, ParameterConfig, SpectralGrid, SpectralModel, initialize, step

    grid = SpectralGrid((2048,))
    model = SpectralModel(grid)
    target = model.render({"centers": torch.tensor([[300.4]], device="cuda")}, torch.ones(1, device="cuda"))
    config = DSFWConfig(coefficients="complex")
    specs = {"centers": ParameterConfig(period=grid.shape)}
    state = initialize(model, target, {"centers": torch.tensor([[900.0]], device="cuda")}, config,
                       candidates={"centers": grid.bins()}, parameters=specs)  # fmt: skip
    assert step(state, config).objective < 0.05 * state.objective


def test_merged_replacement_keeps_each_slot_frozen_components(spectral):
    from dsplat import DSFWConfig, ParameterConfig, initialize
    from dsplat.replacement import merge_support

    model, params, b = spectral
    target = model.render(params, b)
    config = DSFWConfig(coefficients="complex", batch=8, screen_apertures=0)
    specs = {"centers": ParameterConfig(trainable=(True, False), period=model.shape)}
    start = {"centers": torch.tensor([[9.0, 1.0], [14.0, 5.0], [3.0, 11.0]], device="cuda")}
    state = initialize(model, target, start, config, candidates={"centers": model.grid.bins()}, parameters=specs)
    after, replaced = merge_support(state, config, state.candidates)
    assert replaced > 0
    assert torch.equal(after.params["centers"][:, 1], start["centers"][:, 1])
    assert after.objective < state.objective


def test_a_zero_target_fits_with_zero_nmse(spectral):
    from dsplat import DSFWConfig, initialize

    model, params, _ = spectral
    target = torch.zeros(model.shape, dtype=torch.complex64, device="cuda")
    state = initialize(model, target, params, DSFWConfig(coefficients="complex"))
    assert state.history[-1]["nmse"] == 0


def test_range_gate_keeps_points_at_measured_ranges(fmcw):
    model, params, _ = fmcw
    away = params["centers"] + torch.tensor([0, 0, 0.05], device="cuda")
    points = torch.cat((params["centers"], away))
    keep = model.range_gate(points, model.scan.data, 0.1, margin_cells=1.0, min_fraction=0.9)
    assert keep[:5].all() and not keep[5:].any()


def test_certificate_gradient_matches_finite_differences(fmcw):
    from dsplat.certificate import certificate

    model, params, _ = fmcw
    residual = model.scan.data
    probe = {**params, "centers": params["centers"] + 2e-4}
    _, gradient = certificate(model, probe, residual, "real", gradient=True, normals=True)
    for axis in range(3):
        shift = torch.zeros_like(probe["centers"])
        shift[:, axis] = 1e-5
        plus = certificate(model, {**probe, "centers": probe["centers"] + shift}, residual, "real")
        minus = certificate(model, {**probe, "centers": probe["centers"] - shift}, residual, "real")
        numeric = (plus - minus) / 2e-5
        torch.testing.assert_close(gradient[:, axis], numeric, rtol=2e-2,
                                   atol=1e-2 * float(gradient.abs().max()))  # fmt: skip


def test_continuous_refinement_reaches_a_single_reflector(fmcw):
    from dsplat.certificate import CertificateSearchConfig, search_certificate

    model, params, coefficients = fmcw
    one = {k: v[:1] for k, v in params.items()}
    residual = model.render(one, coefficients[:1])
    start = {k: v.repeat(8, *([1] * (v.ndim - 1))) for k, v in one.items()}
    start["centers"] = start["centers"] + 4e-4 * torch.randn_like(start["centers"])
    specs = fmcw_specs()
    params_out, scores = search_certificate(model, residual, start, specs["centers"],
                                            CertificateSearchConfig(peaks=8, separation=0), "real",
                                            normal_spec=specs["normals"])  # fmt: skip
    assert float((params_out["centers"][0] - one["centers"][0]).norm()) < 5e-5
    assert scores[0] > 0.99


def test_spatial_search_proposes_the_true_reflector():
    from dsplat import CertificateSearchConfig, DSFWConfig, FMCWConfig, FMCWModel, Scan, SpatialSearchConfig
    from dsplat import initialize
    from dsplat.spatial import propose

    config = FMCWConfig()
    positions = aperture_grid(8, 0.02)
    truth = surfels(1, seed=5)
    empty = Scan(torch.zeros((64, config.num_range_bins), dtype=torch.complex64, device="cuda"), positions,
                 config)  # fmt: skip
    data = FMCWModel(empty).render(truth, torch.ones(1, device="cuda"))
    model = FMCWModel(Scan(data, positions, config))
    start = {**truth, "normals": torch.tensor([[0.0, 0.0, 1.0]], device="cuda")}
    dsfw_config = DSFWConfig(batch=1)
    state = initialize(model, data, start, dsfw_config, parameters=fmcw_specs())
    search = SpatialSearchConfig(proposal_apertures=64, refine_apertures=0, cache_peaks=0,
                                 continuous=CertificateSearchConfig(peaks=16))  # fmt: skip
    candidates, scores, _ = propose(state, dsfw_config, search)
    assert float((candidates["centers"][0] - truth["centers"][0]).norm()) < 1e-4
    assert math.isfinite(float(scores[0]))


def test_mixed_pooled_statistics_match_the_fp32_stream(fmcw):
    from dsplat import DSFWConfig, initialize
    from dsplat.replacement import pooled_statistics

    model, params, _ = fmcw
    plain, mixed = DSFWConfig(), DSFWConfig(gram="bf16x3", batched=True)
    state = initialize(model, model.scan.data, surfels(5, seed=2), plain, parameters=fmcw_specs())
    pool = {k: torch.cat((v, params[k])) for k, v in state.params.items()}
    gram, rhs = pooled_statistics(state, pool, plain)
    mixed_gram, mixed_rhs = pooled_statistics(state, pool, mixed)
    close(mixed_gram, gram, 1e-4)
    close(mixed_rhs, rhs, 1e-4)
