"""Full-size parity of the splat kernels on the 128^2-array, 2000-surfel sphere cap.

The workload the DSFW metric is quoted on: 16 384 apertures at 2.5 mm pitch, 2000
surfels area-uniform on the front hemisphere of a 30 mm sphere at 0.35 m, 128 range bins.
The GPU kernels run over the whole array; the float64 oracle checks a strided subset of
256 apertures (every 8th per axis), which keeps it to seconds on the CPU.

Tolerances (stated by the workload's correctness bar):
  forward rows        relative L2 <= 1e-5 against the float64 closed form;
  JVP rows, VJP       relative L2 <= 1e-4 against float64 forward / reverse autograd;
  VJP vs central FD   relative L2 <= 1e-4 against float64 central finite differences
                      with h = 1e-7 m on centres (and h = 1e-7 along a tangent for normals).
The upstream of the VJP is zero outside the subset, so the full-array kernel and the
subset oracle compute the same sums.
"""

from __future__ import annotations

import pytest
import torch
from conftest import rel_l2

from oracle import adjoint as oadjoint
from oracle import fmcw as ofmcw

pytestmark = pytest.mark.gpu

FORWARD_TOL = 1e-5
DERIV_TOL = 1e-4
FD_STEP_M = 1e-7
STRIDE = 8


@pytest.fixture(scope="module")
def cap():
    from dsplat import FMCWConfig
    from dsplat.workloads import sphere_cap

    config = FMCWConfig()
    positions, params, reflectivity = sphere_cap(device="cuda")
    weights = (reflectivity * params["areas"].sqrt()).to(torch.complex64)
    generator = torch.Generator().manual_seed(3)
    phases = torch.exp(2j * torch.pi * torch.rand(len(weights), generator=generator, dtype=torch.float64))
    weights = weights * phases.to(torch.complex64).cuda()  # complex weights exercise both parts
    index = torch.arange(16384).reshape(128, 128)[::STRIDE, ::STRIDE].flatten()
    return config, positions, params, weights, index.cuda()


def _oracle_inputs(positions, params, weights, index):
    return (positions[index].cpu(), params["centers"].cpu(), params["normals"].cpu(), weights.cpu())


def test_full_array_forward_rows_within_1e_5_of_float64(cap):
    from dsplat.kernels import surfel as kernel

    config, positions, params, weights, index = cap
    out = kernel.render(config, positions, params["centers"], params["normals"], weights, 0.0)
    assert out.shape == (16384, 128) and out.dtype == torch.complex64
    assert bool(torch.isfinite(torch.view_as_real(out)).all())
    expected = ofmcw.render(config, *_oracle_inputs(positions, params, weights, index))
    assert rel_l2(out[index], expected) < FORWARD_TOL


def _upstream(index, bins, seed=5):
    generator = torch.Generator().manual_seed(seed)
    upstream = torch.zeros((16384, bins), dtype=torch.complex64)
    upstream[index.cpu()] = torch.complex(torch.randn(len(index), bins, generator=generator),
                                          torch.randn(len(index), bins, generator=generator))  # fmt: skip
    return upstream


def test_full_array_vjp_matches_float64_autograd_on_the_subset(cap):
    from dsplat.kernels import surfel as kernel

    config, positions, params, weights, index = cap
    upstream = _upstream(index, config.num_range_bins)
    gc, gn, gw = kernel.vjp(config, positions, params["centers"], params["normals"], weights, upstream.cuda(), 0.0)
    ec, en, ew = ofmcw.vjp(config, *_oracle_inputs(positions, params, weights, index), upstream[index.cpu()])
    assert rel_l2(gc, ec) < DERIV_TOL
    assert rel_l2(gn, en) < DERIV_TOL
    assert rel_l2(gw, ew) < DERIV_TOL


def test_full_array_vjp_matches_the_reference_adjoint_formulas(cap):
    """The CUDA VJP against the reference VJP kernel's own formulas evaluated in float64."""
    from dsplat.kernels import surfel as kernel

    config, positions, params, weights, index = cap
    upstream = _upstream(index, config.num_range_bins, seed=7)
    gc, gn, gw = kernel.vjp(config, positions, params["centers"], params["normals"], weights, upstream.cuda(), 0.0)
    ec, en, ew = oadjoint.vjp(config, *_oracle_inputs(positions, params, weights, index), upstream[index.cpu()])
    assert rel_l2(gc, ec) < DERIV_TOL
    assert rel_l2(gn, en) < DERIV_TOL
    assert rel_l2(gw, ew) < DERIV_TOL


def test_full_array_jvp_rows_match_float64_forward_mode(cap):
    from dsplat.kernels import surfel as kernel

    config, positions, params, weights, index = cap
    generator = torch.Generator().manual_seed(9)
    dc = torch.randn(2000, 3, generator=generator) * 1e-4
    dn = torch.randn(2000, 3, generator=generator) * 1e-2
    dw = weights.cpu() * 0.1
    out = kernel.jvp(config, positions, params["centers"], params["normals"], weights, dc.cuda(), dn.cuda(),
                     dw.cuda(), 0.0)  # fmt: skip
    expected = ofmcw.jvp(config, *_oracle_inputs(positions, params, weights, index), dc, dn, dw)
    assert rel_l2(out[index], expected) < DERIV_TOL


def _surfel_objective(config, positions, center, normal, weight, upstream):
    """Re <upstream, column of one surfel * weight> in float64 (the part of the objective it changes)."""
    column = ofmcw.columns(positions, center[None], normal[None], config)[..., 0]  # [A, K]
    return float((upstream.conj() * column * weight).real.sum())


def test_full_array_vjp_matches_float64_central_differences(cap):
    """Centres by h = 1e-7 m along each axis, normals along one tangent, for eight surfels."""
    from dsplat.kernels import surfel as kernel

    config, positions, params, weights, index = cap
    upstream = _upstream(index, config.num_range_bins, seed=11)
    gc, gn, _ = kernel.vjp(config, positions, params["centers"], params["normals"], weights, upstream.cuda(), 0.0)
    pos = positions[index].cpu().double()
    u = upstream[index.cpu()].to(torch.complex128)
    chosen = torch.linspace(0, 1999, 8).long()
    fd_c, got_c, fd_n, got_n = [], [], [], []
    generator = torch.Generator().manual_seed(13)
    for s in chosen.tolist():
        c = params["centers"][s].cpu().double()
        n = params["normals"][s].cpu().double()
        w = complex(weights[s].cpu())
        for axis in range(3):
            step = torch.zeros(3, dtype=torch.float64)
            step[axis] = FD_STEP_M
            plus = _surfel_objective(config, pos, c + step, n, w, u)
            minus = _surfel_objective(config, pos, c - step, n, w, u)
            fd_c.append((plus - minus) / (2 * FD_STEP_M))
            got_c.append(float(gc[s, axis]))
        tangent = torch.linalg.cross(n, torch.randn(3, generator=generator, dtype=torch.float64))
        tangent = tangent / tangent.norm()
        plus = _surfel_objective(config, pos, c, n + FD_STEP_M * tangent, w, u)
        minus = _surfel_objective(config, pos, c, n - FD_STEP_M * tangent, w, u)
        fd_n.append((plus - minus) / (2 * FD_STEP_M))
        got_n.append(float(gn[s].cpu().double() @ tangent))
    fd_c, got_c = torch.tensor(fd_c), torch.tensor(got_c)
    fd_n, got_n = torch.tensor(fd_n), torch.tensor(got_n)
    assert float(fd_c.abs().max()) > 0 and float(fd_n.abs().max()) > 0
    assert rel_l2(got_c, fd_c) < DERIV_TOL, (got_c, fd_c)
    assert rel_l2(got_n, fd_n) < DERIV_TOL, (got_n, fd_n)
