"""Search kernels and the energy reduction on the GPU against their CPU semantics."""

from __future__ import annotations

import pytest
import torch
from conftest import aperture_grid

from oracle import search as osearch

pytestmark = pytest.mark.gpu


def test_peaks_match_brute_force():
    from dsplat.certificate import select_peaks
    from dsplat.kernels import search

    generator = torch.Generator().manual_seed(1)
    centers = torch.rand(5000, 3, generator=generator)
    scores = torch.rand(5000, generator=generator)
    scores[17] = scores[4]  # a tie keeps the lower index
    for count in (1, 10, 200):
        got = select_peaks(scores.cuda(), centers.cuda(), count, 0.1).cpu()
        assert got.tolist() == osearch.peaks(scores, centers, count, 0.1).tolist()
    scores[::3] = -torch.inf
    got = search.peaks(scores.cuda(), centers.cuda(), 50, 0.05).cpu()
    assert got.tolist() == osearch.peaks(scores, centers, 50, 0.05).tolist()
    assert search.peaks(torch.full((4,), -torch.inf).cuda(), centers[:4].cuda(), 3, 0.1).numel() == 0


def test_range_gate_matches_its_definition():
    from dsplat.kernels import search

    generator = torch.Generator().manual_seed(2)
    positions = aperture_grid(4).cpu()
    points = torch.tensor([0.0, 0.0, 0.3]) + 0.02 * torch.randn(300, 3, generator=generator)
    intervals = (torch.rand(16, 128, generator=generator) > 0.5).int()
    got = search.range_gate(points.cuda(), positions.cuda(), intervals.cuda(), 0.004997, 0.5).cpu()
    assert torch.equal(got, osearch.range_gate(points, positions, intervals, 0.004997, 0.5))


@pytest.mark.parametrize("width", [3, 6])
def test_direction_and_trial_match_their_definition(width):
    from dsplat.kernels import search

    generator = torch.Generator().manual_seed(width)
    count = 37
    m = torch.randn(count, width, width, generator=generator)
    inverse = m @ m.transpose(-1, -2) + 0.1 * torch.eye(width)
    gradient = torch.randn(count, width, generator=generator)
    normals = torch.nn.functional.normalize(torch.randn(count, 3, generator=generator), dim=1)
    mask = torch.tensor([1.0, 1.0, 0.0, 1.0, 1.0, 1.0])
    got = search.direction(inverse.cuda(), gradient.cuda(), normals.cuda(), mask.cuda(), 0.7).cpu()
    expected = osearch.direction(inverse, gradient, normals, mask, 0.7)
    torch.testing.assert_close(got.double(), expected, rtol=1e-5, atol=1e-6)
    centers = torch.randn(count, 3, generator=generator) * 0.01
    controls = torch.tensor([[5e-4] * 3 + [0.1] * 3, [1, 0, 1, 1, 1, 1],
                             [-0.005] * 3 + [0] * 3, [0.005] * 3 + [0] * 3], dtype=torch.float32)  # fmt: skip
    c, n = search.trial(centers.cuda(), normals.cuda(), got.cuda(), controls.cuda(), 0.5)
    ec, en = osearch.trial(centers, normals, got, controls, 0.5)
    torch.testing.assert_close(c.cpu().double(), ec, rtol=1e-6, atol=1e-9)
    torch.testing.assert_close(n.cpu().double(), en, rtol=1e-6, atol=1e-7)


def test_energy_is_exact_and_deterministic():
    from dsplat.kernels.reduce import energy

    generator = torch.Generator().manual_seed(3)
    v = torch.complex(torch.randn(100003, generator=generator), torch.randn(100003, generator=generator))
    r = torch.complex(torch.randn(100003, generator=generator), torch.randn(100003, generator=generator))
    got = energy(v.cuda(), r.cuda())
    assert got.dtype == torch.float64
    torch.testing.assert_close(got.cpu(), osearch.energy(v, r), rtol=1e-12, atol=0)
    assert torch.equal(got, energy(v.cuda(), r.cuda()))
    assert float(energy(v[:0].cuda(), r[:0].cuda())) == 0.0


def test_range_response_matches_the_oracle():
    from dsplat import FMCWConfig
    from dsplat.kernels.response import range_response

    from oracle import fmcw as ofmcw

    config = FMCWConfig()
    got = range_response(config, 62.0, 90.8, 461, "cuda").cpu()
    torch.testing.assert_close(got, ofmcw.range_response(config, 62.0, 90.8, 461), rtol=0, atol=1e-13)


@pytest.mark.parametrize("dimension,separation", [(1, 0.002), (2, 0.03), (3, 0.02), (4, 0.3)])
def test_peaks_in_every_dimension_and_dense_clusters(dimension, separation):
    """Clustered candidates (many suppressed, many taken), up to the 4096-peak limit; one to
    three dimensions look up the taken peaks in the kernel's cell hash, four scan them all."""
    from dsplat.kernels import search

    generator = torch.Generator().manual_seed(dimension)
    seeds = torch.rand(300, dimension, generator=generator)
    centers = seeds[torch.randint(0, 300, (20000,), generator=generator)]
    centers = centers + 0.01 * torch.randn(20000, dimension, generator=generator)
    scores = torch.rand(20000, generator=generator)
    scores[::7] = -torch.inf
    for count in (1, 300, 4096):
        got = search.peaks(scores.cuda(), centers.cuda(), count, separation).cpu()
        assert got.tolist() == osearch.peaks(scores, centers, count, separation).tolist(), count


@pytest.mark.parametrize("mode,fresnel,with_table,bank", [("real", 0.0, True, 24), ("complex", 0.0, True, 24),
                                                         ("real", 1.6, False, 7), ("real", 0.0, True, 0),
                                                         ("complex", 0.0, False, 40)])  # fmt: skip
def test_fused_best_normal_selection_equals_the_scored_selection(mode, fresnel, with_table, bank):
    """orient_candidates with the selection inside the normal-bank launch (dsg_surfel_orient_best)
    against scoring every normal and selecting in PyTorch: the same normal for every candidate
    whose best certificate is not tied to float64 rounding with another normal, and the same
    certificates to float32 rounding; banks of 0 and more than 31 normals, exact bin sums and
    the FFT table, Fresnel."""
    from conftest import aperture_grid, surfels

    from dsplat import FMCWConfig, FMCWModel, Scan
    from dsplat.certificate import orient_candidates

    config = FMCWConfig()
    positions = aperture_grid(12)
    generator = torch.Generator().manual_seed(3)
    residual = torch.complex(torch.randn(len(positions), config.num_range_bins, generator=generator),
                             torch.randn(len(positions), config.num_range_bins, generator=generator)).cuda()  # fmt: skip
    model = FMCWModel(Scan(residual, positions, config), fresnel_n=fresnel)
    params = surfels(3000, seed=4, spread=0.02)
    params["areas"] = params["areas"] * (1 + torch.rand(3000, generator=generator).cuda())
    table = model.range_table(residual, 8) if with_table else None
    scored, scores = orient_candidates(model, params, residual, bank, mode, table)
    fused, fused_scores = orient_candidates(model, params, residual, bank, mode, table, fused=True)
    same = (scored["normals"] == fused["normals"]).all(1)
    assert float(same.float().mean()) > 0.999, float(same.float().mean())
    torch.testing.assert_close(fused_scores[same], scores[same], rtol=1e-6, atol=0)
