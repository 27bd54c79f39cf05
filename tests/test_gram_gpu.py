"""tcgen05 split-BF16x3 Gram against float64 products (parity tests)."""

from __future__ import annotations

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n", [(64, 128), (3000, 300), (20000, 1000)])
def test_split_bf16x3_gram_matches_float64(m, n):
    from dsplat.kernels.gram import GramRows

    generator = torch.Generator().manual_seed(m + n)
    rows = torch.randn(m, n, generator=generator) * (1 + torch.rand(n, generator=generator))
    rows = rows.cuda()
    total = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    store = GramRows(n, m, "cuda")
    half = m // 2
    store.append(rows[:half])
    store.append(rows[half:])
    status = store.accumulate(total)
    assert int(status.item()) == 0
    expected = rows.double().T @ rows.double()
    upper = torch.triu(torch.ones(n, n, dtype=torch.bool, device="cuda"))
    error = (total - expected)[upper].abs().max() / expected.abs().max()
    assert float(error) < 3e-5, float(error)
    # The strict lower triangle of off-diagonal tiles is never written.
    if n > 128:
        assert float(total[200:, :128].abs().max()) == 0.0


@pytest.mark.parametrize("splits", [1, 3, 8])
def test_k_split_gram_is_bitwise_reproducible_and_split_independent(splits):
    """The K-split parts are added in split order by a second kernel (no atomics): two runs
    give identical bits. Each split accumulates its share of the 625 stages in FP32 tensor
    memory, so one split over all 40 000 rows is the least accurate (about 3e-4 of the
    largest entry against float64); more splits shorten the FP32 sums."""
    from dsplat.kernels.gram import GramRows

    generator = torch.Generator().manual_seed(11)
    rows = (torch.randn(40000, 700, generator=generator) * (1 + torch.rand(700, generator=generator))).cuda()
    store = GramRows(700, len(rows), "cuda")
    store.append(rows)
    results = []
    for count in (splits, splits, 1):
        total = torch.zeros((700, 700), dtype=torch.float64, device="cuda")
        assert int(store.accumulate(total, splits=count).item()) == 0
        results.append(total)
    assert torch.equal(results[0], results[1])
    expected = rows.double().T @ rows.double()
    upper = torch.triu(torch.ones(700, 700, dtype=torch.bool, device="cuda"))
    errors = [float((total - expected)[upper].abs().max() / expected.abs().max()) for total in results]
    assert max(errors) < 1e-3, errors
    if splits > 1:
        assert errors[0] <= errors[2] * 1.01, errors


def test_bf16x3_is_far_more_accurate_than_one_bf16_pass():
    from dsplat.kernels.gram import GramRows

    generator = torch.Generator().manual_seed(3)
    rows = torch.randn(4096, 256, generator=generator).cuda()
    total = torch.zeros((256, 256), dtype=torch.float64, device="cuda")
    store = GramRows(256, 4096, "cuda")
    store.append(rows)
    store.accumulate(total)
    expected = rows.double().T @ rows.double()
    single = rows.bfloat16().double().T @ rows.bfloat16().double()
    upper = torch.triu(torch.ones(256, 256, dtype=torch.bool, device="cuda"))
    err3 = float((total - expected)[upper].abs().max())
    err1 = float((single - expected)[upper].abs().max())
    # FP32 accumulation in TMEM dominates what remains of the split-BF16x3 error.
    assert err3 < err1 / 10


def test_column_range_gram_covers_the_new_columns():
    from dsplat.kernels.gram import GramRows

    generator = torch.Generator().manual_seed(9)
    m, n, start = 5000, 700, 450
    rows = torch.randn(m, n, generator=generator).cuda()
    total = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    store = GramRows(n, m, "cuda")
    store.append(rows)
    assert int(store.accumulate(total, column_from=start).item()) == 0
    expected = rows.double().T @ rows.double()
    i, j = torch.meshgrid(torch.arange(n), torch.arange(n), indexing="ij")
    needed = ((i <= j) & (j >= start)).cuda()
    error = (total - expected)[needed].abs().max() / expected.abs().max()
    assert float(error) < 3e-5
    assert float(total[:, : start - 128].abs().max()) == 0.0  # columns of earlier tiles untouched


def test_emulated_projection_is_fp32_accurate():
    from dsplat.kernels.gemm import emulated, project

    generator = torch.Generator().manual_seed(10)
    matrix = torch.randn(60, 256, generator=generator).cuda()
    rows = torch.randn(256, 40000, generator=generator).cuda()
    with emulated():
        fast = project(matrix, rows)
    exact = matrix.double() @ rows.double()
    assert float((fast.double() - exact).abs().max() / exact.abs().max()) < 1e-5


@pytest.mark.parametrize("pad", [2, 4])
def test_fused_design_projection_gram_matches_the_fp32_stream(pad):
    """Normal equations from on-chip dictionary rows (tcgen05 projection + Gram) vs the FP32 path."""
    from dsplat import DSFWConfig, FMCWConfig, FMCWModel, ParameterConfig, Scan
    from dsplat.varpro import normal_equations
    from dsplat.workloads import box_of, sphere_cap

    config = FMCWConfig(pad_factor=pad) if pad == 2 else FMCWConfig(pad_factor=pad, adc_samples=64)
    positions, params, reflectivity = sphere_cap(surfel_count=300, side=24, device="cuda")
    data = FMCWModel(Scan(torch.zeros((len(positions), config.num_range_bins), dtype=torch.complex64,
                                      device="cuda"), positions, config)).render(params, reflectivity)
    low, high = box_of(params["centers"])
    specs = {"centers": ParameterConfig(lower=low, upper=high)}
    model = FMCWModel(Scan(data, positions, config)).prepare(specs)
    plain = normal_equations(model, params, data, DSFWConfig(row_chunk=8 * config.num_range_bins))
    mixed = normal_equations(model, params, data, DSFWConfig(row_chunk=8 * config.num_range_bins, gram="bf16x3"))
    scale = float(plain[0].abs().max())
    assert float((mixed[0] - plain[0]).abs().max()) < 1e-4 * scale
    assert float((mixed[1] - plain[1]).abs().max()) < 1e-4 * float(plain[1].abs().max())


@pytest.mark.parametrize("pad,rank2,surfels", [(2, 56, 300), (2, 2, 1), (4, 100, 129), (1, 128, 257), (2, 34, 128)])
def test_design_projection_matches_float64(pad, rank2, surfels):
    """dsg_design_project_bf16x3 straight through the C ABI against the float64 oracle:
    PT[s, offset + a rank2 + rho] = sum_j U[rho, j] v_{a,s}[j], v the real dictionary row
    (re, im interleaved per bin) including sqrt(area). Partial tiles, ranks that are not a
    multiple of 32 and a nonzero column offset all appear."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    from conftest import aperture_grid, surfels as make_surfels
    from dsplat import FMCWConfig
    from dsplat.kernels import _lib
    from dsplat.kernels.gram import split_basis

    from oracle import fmcw as ofmcw

    config = FMCWConfig(pad_factor=pad, adc_samples=256 // pad)  # 128 range bins
    K = config.num_range_bins
    positions = aperture_grid(6)
    params = make_surfels(surfels, seed=rank2)
    A = len(positions)
    generator = torch.Generator().manual_seed(rank2 + surfels)
    basis = (torch.randn(rank2, 2 * K, generator=generator) / (2 * K) ** 0.5).cuda()
    hi_u, lo_u = split_basis(basis)
    offset = 6
    ld = offset + A * rank2 + 4
    pt_hi = torch.zeros((surfels, ld), dtype=torch.bfloat16, device="cuda")
    pt_lo = torch.zeros_like(pt_hi)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("dsg_design_project_bf16x3", _lib.chirp(config, 0.0), _lib.ptr(positions), A,
              _lib.ptr(params["centers"]), _lib.ptr(params["normals"]), _lib.ptr(params["areas"]), surfels,
              _lib.ptr(hi_u), _lib.ptr(lo_u), rank2, _lib.ptr(pt_hi), _lib.ptr(pt_lo), ld, offset,
              _lib.ptr(status), _lib.stream(positions.device))  # fmt: skip
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = (pt_hi.double() + pt_lo.double()).cpu()
    rows = ofmcw.design(config, positions.cpu(), params["centers"].cpu(), params["normals"].cpu(),
                        params["areas"].cpu(), real=True)  # [2K A, S], row j A + a
    v = rows.reshape(2 * K, A, surfels)
    expected = torch.einsum("rj,jas->sar", basis.cpu().double(), v).reshape(surfels, A * rank2)
    block = got[:, offset : offset + A * rank2]
    scale = float(expected.abs().max())
    assert float((block - expected).abs().max()) < 5e-5 * scale
    assert float((block - expected).norm() / expected.norm()) < 2e-5
    # Columns outside the block are never written.
    assert float(got[:, :offset].abs().max()) == 0.0 and float(got[:, offset + A * rank2 :].abs().max()) == 0.0
