"""The oracle against golden vectors of the reference's own float64 oracles (CPU).

tests/golden/reference_oracles.npz was produced by tests/golden/make_golden.py from
the reference's tests/reference/kernel.py, tests/reference/oracle.py and
dsplat/groundtruth.py; agreement here pins oracle/ before it checks any kernel.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import fmcw as ofmcw
from oracle import kernel as okernel
from oracle import spectral as ospectral

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_oracles.npz")


def _cfg(**kw):
    from dsplat import FMCWConfig

    return FMCWConfig(**kw)


def test_dirichlet_and_windows_match_the_reference_oracle():
    delta = torch.from_numpy(GOLDEN["delta"])
    for samples, n_fft in ((128, 256), (128, 512), (24, 24), (16, 24)):
        value, deriv = okernel.dirichlet(delta, samples, n_fft)
        expected = torch.from_numpy(GOLDEN[f"dirichlet_{samples}_{n_fft}"])
        torch.testing.assert_close(value, expected[0], rtol=0, atol=1e-12)
        torch.testing.assert_close(deriv, expected[1], rtol=0, atol=1e-12)
    for window, samples, n_fft, beta in (("hann", 20, 24, 14.0), ("hamming", 16, 24, 14.0),
                                         ("kaiser", 12, 16, 6.0)):  # fmt: skip
        value, deriv = okernel.windowed(delta, samples, n_fft, window, beta)
        expected = torch.from_numpy(GOLDEN[f"window_{window}_{samples}_{n_fft}"])
        torch.testing.assert_close(value, expected[0], rtol=0, atol=1e-12)
        torch.testing.assert_close(deriv, expected[1], rtol=0, atol=1e-10)


@pytest.mark.parametrize("name,pad,fresnel", [("pad2", 2, 0.0), ("pad4", 4, 0.0), ("fresnel", 2, 1.6)])
def test_fmcw_columns_match_the_reference_oracle(name, pad, fresnel):
    positions = torch.from_numpy(GOLDEN["fmcw_positions"])
    centers = torch.from_numpy(GOLDEN["fmcw_centers"])
    normals = torch.from_numpy(GOLDEN["fmcw_normals"])
    cols = ofmcw.columns(positions, centers, normals, _cfg(pad_factor=pad), fresnel)
    expected = torch.from_numpy(GOLDEN[f"fmcw_columns_{name}"])
    torch.testing.assert_close(cols, expected, rtol=0, atol=1e-12 * float(expected.abs().max()))


@pytest.mark.parametrize("name,pad", [("pad2", 2), ("pad4", 4)])
def test_adc_synthesis_matches_the_reference(name, pad):
    args = [torch.from_numpy(GOLDEN[f"synth_{k}"]) for k in ("positions", "centers", "normals", "amplitudes")]
    scan = ofmcw.synthesize(*args, _cfg(pad_factor=pad))
    expected = torch.from_numpy(GOLDEN[f"synth_{name}"]).to(torch.complex128)
    # The reference stores complex64.
    torch.testing.assert_close(scan, expected, rtol=0, atol=1e-6 * float(expected.abs().max()))


def test_planar_arrays_match_the_reference():
    from dsplat.groundtruth import planar_array

    for name, axis in (("z", (0, 0, 1)), ("x", (1, 0, 0)), ("negz", (0, 0, -1)), ("skew", (0.3, -0.2, 1))):
        torch.testing.assert_close(planar_array(5, 0.003, axis=axis),
                                   torch.from_numpy(GOLDEN[f"planar_{name}"]))  # fmt: skip


@pytest.mark.parametrize("name", ["rect32", "hann24x20", "hamming24x20", "kaiser16x12", "radius24x20"])
def test_spectral_dictionaries_match_the_reference_oracle(name):
    from dsplat import SpectralGrid

    grids = {
        "rect32": SpectralGrid((32,)),
        "hann24x20": SpectralGrid((24, 20), window="hann"),
        "hamming24x20": SpectralGrid((24, 20), samples=(16, 20), window="hamming"),
        "kaiser16x12": SpectralGrid((16, 12), window="kaiser", beta=6.0),
        "radius24x20": SpectralGrid((24, 20), radius=4.0),
    }
    grid = grids[name]
    centers = torch.from_numpy(GOLDEN[f"spectral_{name}_centers"])
    a, da = ospectral.design(grid, centers, grid.bins("cpu"))
    torch.testing.assert_close(a, torch.from_numpy(GOLDEN[f"spectral_{name}_a"]), rtol=0, atol=1e-12)
    torch.testing.assert_close(da, torch.from_numpy(GOLDEN[f"spectral_{name}_da"]), rtol=0, atol=1e-10)


def test_oracle_derivatives_agree_with_central_differences():
    """The autograd VJP of the oracle matches float64 central differences (h = 1e-7 m)."""
    config = _cfg()
    positions = torch.from_numpy(GOLDEN["fmcw_positions"]).double()
    centers = torch.from_numpy(GOLDEN["fmcw_centers"]).double()
    normals = torch.from_numpy(GOLDEN["fmcw_normals"]).double()
    weights = torch.tensor([1.0, -0.5, 0.7, 0.2, 1.1], dtype=torch.complex128) * 0.01
    generator = torch.Generator().manual_seed(2)
    upstream = torch.randn(len(positions), config.num_range_bins, dtype=torch.complex128, generator=generator)
    gc, gn, gw = ofmcw.vjp(config, positions, centers, normals, weights, upstream)
    h = 1e-7

    def objective(c, n):
        return float((upstream.conj() * ofmcw.render(config, positions, c, n, weights)).real.sum())

    for axis in range(3):
        shift = torch.zeros_like(centers)
        shift[:, axis] = h
        for s in range(len(centers)):
            plus, minus = centers.clone(), centers.clone()
            plus[s] += shift[s]
            minus[s] -= shift[s]
            numeric = (objective(plus, normals) - objective(minus, normals)) / (2 * h)
            assert abs(numeric - float(gc[s, axis])) <= 1e-4 * float(gc.abs().max())


def test_scene_oracle_matches_the_reference_physics_renderer():
    """oracle.scene against tests/reference/physics.py (values and autograd gradients)."""
    from dsplat.spectral import SpectralGrid
    from dsplat.surfel import Sensor

    from oracle import scene

    golden = np.load(Path(__file__).parent / "golden" / "reference_scene.npz")
    keys = ("positions", "normals", "areas", "reflectivity", "velocities", "impedance")
    for name, shape, window in (("rect", (32, 16, 8), "rect"), ("hann", (24, 12, 6), "hann")):
        inputs = [torch.from_numpy(golden[f"{name}_{k}"]).requires_grad_() for k in keys]
        gamma = float(golden[f"{name}_meta"][0])
        sensor = Sensor(shape=shape)
        cube = scene.render_scene(*inputs, sensor, SpectralGrid(shape, window=window), gamma=gamma)
        expected = torch.from_numpy(golden[f"{name}_cube"])
        assert float((cube.detach() - expected).abs().max() / expected.abs().max()) < 1e-12
        upstream = torch.from_numpy(golden[f"{name}_upstream"])
        grads = torch.autograd.grad((upstream.conj() * cube).real.sum(), inputs)
        for key, grad in zip(keys, grads, strict=True):
            ref = torch.from_numpy(golden[f"{name}_grad_{key}"])
            assert float((grad - ref).abs().max() / ref.abs().max().clamp(min=1e-300)) < 1e-10, key
