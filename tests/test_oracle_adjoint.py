"""The float64 restatement of the reference's hand-derived adjoint against oracle autograd (CPU).

oracle/adjoint.py evaluates the reference VJP kernel's own formulas (per-class cotangent
sums, the nearest bin evaluated directly, the chain rule through range, obliquity and
carrier; dsplat/kernels/surfel.slang:227-311) in float64. Autograd of the closed form
(oracle/fmcw.py) is a separate derivation; the two must agree to float64 rounding, which
pins the adjoint formulas before the GPU tests compare the CUDA VJP with them.
"""

from __future__ import annotations

import pytest
import torch

from oracle import adjoint as oadjoint
from oracle import fmcw as ofmcw


def _cfg(**kw):
    from dsplat import FMCWConfig

    return FMCWConfig(**kw)


def _case(side, count, seed):
    from conftest import aperture_grid, surfels

    positions = aperture_grid(side, device="cpu").double()
    params = surfels(count, seed=seed, device="cpu")
    generator = torch.Generator().manual_seed(seed + 11)
    weights = torch.complex(torch.randn(count, generator=generator, dtype=torch.float64),
                            torch.randn(count, generator=generator, dtype=torch.float64)) * 1e-2  # fmt: skip
    return positions, params["centers"].double(), params["normals"].double(), weights, generator


def _rel(a, b):
    return float((a - b).norm() / b.norm())


@pytest.mark.parametrize("pad,fresnel", [(2, 0.0), (4, 0.0), (2, 1.6), (1, 0.0)])
def test_adjoint_formulas_equal_autograd_of_the_closed_form(pad, fresnel):
    config = _cfg(pad_factor=pad) if pad != 1 else _cfg(pad_factor=1, adc_samples=256)
    positions, centers, normals, weights, generator = _case(5, 6, seed=pad)
    bins = config.num_range_bins
    upstream = torch.complex(torch.randn(len(positions), bins, generator=generator, dtype=torch.float64),
                             torch.randn(len(positions), bins, generator=generator, dtype=torch.float64))  # fmt: skip
    ac, an, aw = oadjoint.vjp(config, positions, centers, normals, weights, upstream, fresnel)
    ec, en, ew = ofmcw.vjp(config, positions, centers, normals, weights, upstream, fresnel)
    assert _rel(ac, ec) < 1e-11
    assert _rel(an, en) < 1e-11
    assert _rel(aw, ew) < 1e-11


def test_adjoint_formulas_on_and_next_to_a_bin():
    """Peaks exactly on a bin, a hair off it and half way between: the nearest-bin path."""
    config = _cfg()
    positions, centers, normals, weights, generator = _case(3, 4, seed=9)
    spacing = config.range_bin_spacing_m
    p0 = positions[0]
    for s, frac in ((0, 0.0), (1, 1e-6), (2, 0.5), (3, -0.49)):
        r = (p0 - centers[s]).norm()
        target = (torch.round(r / spacing) + frac) * spacing
        centers[s] = p0 + (centers[s] - p0) * target / r
    upstream = torch.complex(torch.randn(len(positions), config.num_range_bins, generator=generator,
                                         dtype=torch.float64),
                             torch.randn(len(positions), config.num_range_bins, generator=generator,
                                         dtype=torch.float64))  # fmt: skip
    ac, an, aw = oadjoint.vjp(config, positions, centers, normals, weights, upstream)
    ec, en, ew = ofmcw.vjp(config, positions, centers, normals, weights, upstream)
    assert _rel(ac, ec) < 1e-8 and _rel(an, en) < 1e-8 and _rel(aw, ew) < 1e-11


def test_back_facing_pairs_contribute_nothing():
    config = _cfg()
    positions, centers, normals, weights, generator = _case(3, 3, seed=2)
    normals = -normals  # every surfel faces away from the apertures
    upstream = torch.ones(len(positions), config.num_range_bins, dtype=torch.complex128)
    ac, an, aw = oadjoint.vjp(config, positions, centers, normals, weights, upstream)
    assert float(ac.abs().max()) == 0.0 and float(an.abs().max()) == 0.0 and float(aw.abs().max()) == 0.0
