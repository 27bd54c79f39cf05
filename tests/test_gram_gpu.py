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
