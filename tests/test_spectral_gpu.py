"""Spectral atoms on the GPU against the float64 oracle, and one linear map (parity tests)."""

from __future__ import annotations

import pytest
import torch
from conftest import close, rel_l2

from oracle import spectral as ospectral

pytestmark = pytest.mark.gpu


def _grids():
    from dsplat import SpectralGrid

    return [
        SpectralGrid((32,)),
        SpectralGrid((24, 20), window="hann"),
        SpectralGrid((24, 20), samples=(16, 20), window="hamming"),
        SpectralGrid((16, 12), window="kaiser", beta=6.0),
        SpectralGrid((24, 20), radius=4.0),
        SpectralGrid((8, 6, 5)),
        SpectralGrid((256, 256)),
    ]


@pytest.mark.parametrize("index", range(7))
def test_design_matches_the_oracle(index):
    from dsplat.kernels import spectral as kernel

    grid = _grids()[index]
    generator = torch.Generator().manual_seed(index)
    count = 7 if grid.size < 10000 else 3
    centers = (torch.rand(count, len(grid.shape), generator=generator) * torch.tensor(grid.shape)).cuda()
    bins = grid.bins()
    a, da = kernel.design(grid, centers, bins, derivatives=True)
    ea, eda = ospectral.design(grid, centers, bins)
    if grid.radius:  # the truncated kernel is discontinuous at the support boundary
        inside = (ea.abs() > 0)[..., None]
        eda, da = eda * inside, da * inside.to(da.device)
    close(a, ea, 2e-6)
    close(da, eda, 1e-5)


def test_render_jvp_and_vjp_are_one_linear_map(spectral):
    from dsplat.kernels import spectral as kernel

    model, params, b = spectral
    grid, centers = model.grid, params["centers"]
    bins = grid.bins()
    a, da = ospectral.design(grid, centers, bins)
    assert rel_l2(kernel.render(grid, centers, b, bins), a @ b.cpu().to(torch.complex128)) < 1e-5
    generator = torch.Generator().manual_seed(3)
    dc = torch.randn(centers.shape, generator=generator).cuda()
    db = torch.complex(torch.randn(3, generator=generator), torch.randn(3, generator=generator)).cuda()
    jvp = kernel.jvp(grid, centers, b, dc, db, bins)
    assert rel_l2(jvp, ospectral.jvp(grid, centers, b, dc, db, bins)) < 1e-5
    upstream = torch.complex(torch.randn(len(bins), generator=generator),
                             torch.randn(len(bins), generator=generator)).cuda()  # fmt: skip
    gc, gb = kernel.vjp(grid, centers, b, upstream, bins)
    ec, eb = ospectral.vjp(grid, centers, b, upstream, bins)
    assert rel_l2(gc, ec) < 1e-5 and rel_l2(gb, eb) < 1e-5
    left = (upstream.conj() * jvp).real.sum().double()
    right = (gc.double() * dc.double()).sum() + (gb.conj() * db).real.sum().double()
    torch.testing.assert_close(left, right, rtol=1e-5, atol=1e-6)
    centers_leaf, b_leaf = centers.clone().requires_grad_(), b.clone().requires_grad_()
    (upstream.conj() * kernel.render(grid, centers_leaf, b_leaf, bins)).real.sum().backward()
    close(centers_leaf.grad, gc, 1e-6)
    close(b_leaf.grad, gb, 1e-6)


def test_star_workload_forward_is_within_1e_5():
    from dsplat import SpectralGrid
    from dsplat.kernels import spectral as kernel
    from dsplat.workloads import star_tones

    target, truth = star_tones()
    grid = SpectralGrid((256, 256))
    generator = torch.Generator().manual_seed(0)
    b = torch.polar(torch.ones(80), 6.28 * torch.rand(80, generator=generator)).cuda()
    bins = grid.bins()
    out = kernel.render(grid, truth, b, bins)
    a, _ = ospectral.design(grid, truth, bins)
    assert rel_l2(out, a @ b.cpu().to(torch.complex128)) < 1e-5


@pytest.mark.parametrize("index", range(7))
def test_whole_grid_products_from_axis_tables_match_the_oracle(index):
    """The separable path of the spectral model (per-axis tables, complex products):
    forward, JVP and VJP on the whole grid against the float64 oracle, the adjoint
    identity, and autograd through the grid forward equal to the hand-written adjoint."""
    from dsplat.kernels import spectral as kernel

    grid = _grids()[index]
    generator = torch.Generator().manual_seed(10 + index)
    count = 7 if grid.size < 10000 else 80
    centers = (torch.rand(count, len(grid.shape), generator=generator) * torch.tensor(grid.shape)).cuda()
    b = torch.complex(torch.randn(count, generator=generator), torch.randn(count, generator=generator)).cuda()
    bins = grid.bins()
    a, _ = ospectral.design(grid, centers, bins)
    out = kernel.render_grid(grid, centers, b)
    assert out.shape == (grid.size,)
    assert rel_l2(out, a @ b.cpu().to(torch.complex128)) < 1e-5
    dc = torch.randn(centers.shape, generator=generator).cuda()
    db = torch.complex(torch.randn(count, generator=generator), torch.randn(count, generator=generator)).cuda()
    jvp = kernel.jvp_grid(grid, centers, b, dc, db)
    expected_jvp = ospectral.jvp(grid, centers, b, dc, db, bins)
    upstream = torch.complex(torch.randn(grid.size, generator=generator),
                             torch.randn(grid.size, generator=generator)).cuda()  # fmt: skip
    gc, gb = kernel.vjp_grid(grid, centers, b, upstream)
    ec, eb = ospectral.vjp(grid, centers, b, upstream, bins)
    if grid.radius:  # the truncated kernel's derivative jumps at the support edge; compare the values only
        assert rel_l2(gb, eb) < 1e-5
    else:
        assert rel_l2(jvp, expected_jvp) < 1e-5
        assert rel_l2(gc, ec) < 1e-5 and rel_l2(gb, eb) < 1e-5
    left = (upstream.conj() * jvp).real.sum().double()
    right = (gc.double() * dc.double()).sum() + (gb.conj() * db).real.sum().double()
    torch.testing.assert_close(left, right, rtol=1e-4, atol=1e-5)
    centers_leaf, b_leaf = centers.clone().requires_grad_(), b.clone().requires_grad_()
    (upstream.conj() * kernel.render_on_grid(grid, centers_leaf, b_leaf)).real.sum().backward()
    close(centers_leaf.grad, gc, 1e-6)
    close(b_leaf.grad, gb, 1e-6)
