"""Generate the golden vectors that pin the oracle against the reference itself.

Run here, where the reference checkout exists (it never exists on the GPU machine):

    python tests/golden/make_golden.py /path/to/Dirichlet-Splatting   (or set DSPLAT_REFERENCE)

It imports the reference's own float64 oracles (tests/reference/kernel.py,
tests/reference/oracle.py, tests/reference/physics.py, dsplat/groundtruth.py and the
pure-torch dsplat/fmcw.py migration) with a stub
`slangtorch` module,
evaluates them on seeded inputs and writes the inputs and outputs to
tests/golden/reference_oracles.npz. tests/test_oracle_golden.py then checks the
repository's oracle/ against these vectors. The reference's Slang kernels are not
run (slangtorch and a GPU are unavailable here).
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent


def reference_root(args):
    """The reference checkout: the first argument, else $DSPLAT_REFERENCE; there is no default."""
    import os

    value = args[0] if args else os.environ.get("DSPLAT_REFERENCE")
    if not value:
        raise SystemExit("name the reference checkout: an argument or DSPLAT_REFERENCE=/path/to/Dirichlet-Splatting")
    root = Path(value)
    if not (root / "dsplat").is_dir():
        raise SystemExit(f"{root} holds no dsplat package")
    return root


def import_reference(root: Path):
    """Import the reference's pure-torch oracles with a stub slangtorch."""
    sys.modules.setdefault("slangtorch", types.ModuleType("slangtorch"))
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import dsplat.groundtruth as groundtruth  # noqa: E402
    import reference.kernel as kernel  # noqa: E402
    import reference.oracle as oracle  # noqa: E402
    from dsplat import FMCWConfig, SpectralGrid  # noqa: E402

    return groundtruth, kernel, oracle, FMCWConfig, SpectralGrid


def aperture_grid(side, pitch):
    t = (torch.arange(side, dtype=torch.float32) - (side - 1) / 2) * pitch
    x, y = torch.meshgrid(t, t, indexing="ij")
    return torch.stack([x.flatten(), y.flatten(), torch.zeros(side * side)], -1)


def surfels(count, seed, spread=0.01):
    generator = torch.Generator().manual_seed(seed)
    centers = torch.tensor([0, 0, 0.3]) + spread * (2 * torch.rand(count, 3, generator=generator) - 1)
    direction = torch.tensor([0.0, 0, -1]) + 0.3 * torch.randn(count, 3, generator=generator)
    normals = torch.nn.functional.normalize(direction, dim=1)
    return centers.float(), normals.float()


def main(root: Path) -> None:
    groundtruth, kernel, oracle, FMCWConfig, SpectralGrid = import_reference(root)
    out: dict[str, np.ndarray] = {}

    # Dirichlet kernel and windows on deltas that cross the Taylor branch and the wrap.
    generator = torch.Generator().manual_seed(11)
    delta = torch.cat([
        torch.linspace(-300.0, 300.0, 1201, dtype=torch.float64),
        (torch.rand(400, generator=generator, dtype=torch.float64) - 0.5) * 4e-3,
        torch.tensor([0.0, 1e-4, -1e-4, 0.5, -0.5, 127.0, 128.0, 255.9], dtype=torch.float64),
    ])
    out["delta"] = delta.numpy()
    for samples, n_fft in ((128, 256), (128, 512), (24, 24), (16, 24)):
        value, deriv = kernel.dirichlet(delta, samples, n_fft)
        out[f"dirichlet_{samples}_{n_fft}"] = torch.stack([value, deriv]).numpy()
    for window, samples, n_fft, beta in (("hann", 20, 24, 14.0), ("hamming", 16, 24, 14.0),
                                         ("kaiser", 12, 16, 6.0)):  # fmt: skip
        value, deriv = kernel.windowed_kernel(delta, samples, n_fft, window, beta)
        out[f"window_{window}_{samples}_{n_fft}"] = torch.stack([value, deriv]).numpy()

    # FMCW columns (float64 closed form) for two chirps and a dielectric.
    positions = aperture_grid(4, 0.008)
    centers, normals = surfels(5, 0)
    out["fmcw_positions"], out["fmcw_centers"], out["fmcw_normals"] = (
        positions.numpy(), centers.numpy(), normals.numpy())  # fmt: skip
    for name, config, fresnel in (("pad2", FMCWConfig(), 0.0), ("pad4", FMCWConfig(pad_factor=4), 0.0),
                                  ("fresnel", FMCWConfig(), 1.6)):  # fmt: skip
        out[f"fmcw_columns_{name}"] = oracle.fmcw_columns(positions, centers, normals, config, fresnel).numpy()

    # ADC-domain synthesis (independent of the Dirichlet kernel).
    positions6 = aperture_grid(4, 0.006)
    centers4, normals4 = surfels(4, 3)
    amplitudes = torch.linspace(0.5, 1.5, 4) * 0.01
    out["synth_positions"], out["synth_centers"], out["synth_normals"], out["synth_amplitudes"] = (
        positions6.numpy(), centers4.numpy(), normals4.numpy(), amplitudes.numpy())  # fmt: skip
    for name, config in (("pad2", FMCWConfig()), ("pad4", FMCWConfig(pad_factor=4))):
        scan = groundtruth.synthesize(positions6, centers4, normals4, amplitudes, config)
        out[f"synth_{name}"] = scan.data.numpy()

    # Planar arrays facing several axes.
    for name, axis in (("z", (0, 0, 1)), ("x", (1, 0, 0)), ("negz", (0, 0, -1)), ("skew", (0.3, -0.2, 1))):
        out[f"planar_{name}"] = groundtruth.planar_array(5, 0.003, axis=axis).numpy()

    # Spectral dictionaries of the reference's own test grids.
    grids = {
        "rect32": SpectralGrid((32,)),
        "hann24x20": SpectralGrid((24, 20), window="hann"),
        "hamming24x20": SpectralGrid((24, 20), samples=(16, 20), window="hamming"),
        "kaiser16x12": SpectralGrid((16, 12), window="kaiser", beta=6.0),
        "radius24x20": SpectralGrid((24, 20), radius=4.0),
    }
    generator = torch.Generator().manual_seed(5)
    for name, grid in grids.items():
        centers_s = torch.rand(7, len(grid.shape), generator=generator) * torch.tensor(grid.shape)
        bins = grid.bins("cpu")
        a, da = oracle.spectral_design(grid, centers_s, bins)
        out[f"spectral_{name}_centers"] = centers_s.numpy()
        out[f"spectral_{name}_a"] = a.numpy()
        out[f"spectral_{name}_da"] = da.numpy()

    np.savez_compressed(HERE / "reference_oracles.npz", **out)
    print("wrote", HERE / "reference_oracles.npz", sum(v.nbytes for v in out.values()) // 1024, "KiB")


def scene_inputs(count=6, seed=3):
    """Seeded 13-DOF surfels in front of a range/Doppler/azimuth sensor at the origin."""
    g = torch.Generator().manual_seed(seed)
    positions = torch.tensor([0.0, 0.0, 1.5]) + 0.3 * torch.randn(count, 3, generator=g, dtype=torch.float64)
    normals = torch.nn.functional.normalize(-positions + 0.2 * torch.randn(count, 3, generator=g, dtype=torch.float64),
                                            dim=1)  # fmt: skip
    areas = 1e-3 * (1 + torch.rand(count, generator=g, dtype=torch.float64))
    reflectivity = torch.complex(torch.rand(count, generator=g, dtype=torch.float64),
                                 torch.rand(count, generator=g, dtype=torch.float64))  # fmt: skip
    velocities = torch.randn(count, 3, generator=g, dtype=torch.float64)
    impedance = torch.complex(1 + torch.rand(count, generator=g, dtype=torch.float64),
                              0.1 * torch.rand(count, generator=g, dtype=torch.float64))  # fmt: skip
    return positions, normals, areas, reflectivity, velocities, impedance


def scene_cases(root: Path) -> None:
    """The reference's float64 composed renderer (tests/reference/physics.py) and the
    gradients of Re(conj(u) . cube) by autograd, written to reference_scene.npz."""
    sys.modules.setdefault("slangtorch", types.ModuleType("slangtorch"))
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import reference.physics as physics  # noqa: E402
    from dsplat.surfel import Sensor  # noqa: E402

    out: dict[str, np.ndarray] = {}
    for name, shape, window, gamma in (("rect", (32, 16, 8), "rect", 1.0), ("hann", (24, 12, 6), "hann", 2.0)):
        inputs = [x.clone().requires_grad_() for x in scene_inputs(seed=len(out) + 3)]
        sensor = Sensor(shape=shape)
        cube = physics.render_scene(*inputs, sensor, window=window, gamma=gamma)
        g = torch.Generator().manual_seed(7)
        upstream = torch.complex(torch.randn(shape, generator=g, dtype=torch.float64),
                                 torch.randn(shape, generator=g, dtype=torch.float64))  # fmt: skip
        grads = torch.autograd.grad((upstream.conj() * cube).real.sum(), inputs)
        keys = ("positions", "normals", "areas", "reflectivity", "velocities", "impedance")
        for key, value, grad in zip(keys, inputs, grads, strict=True):
            out[f"{name}_{key}"] = value.detach().numpy()
            out[f"{name}_grad_{key}"] = grad.numpy()
        out[f"{name}_upstream"] = upstream.numpy()
        out[f"{name}_cube"] = cube.detach().numpy()
        out[f"{name}_meta"] = np.array([gamma])
    np.savez_compressed(HERE / "reference_scene.npz", **out)
    print("wrote", HERE / "reference_scene.npz")


def migration_cases(root: Path) -> None:
    """The reference's range-migration initializer (dsplat/fmcw.py:361-454, pure torch) on
    scans synthesized by its own groundtruth.synthesize, written to reference_migration.npz."""
    sys.modules.setdefault("slangtorch", types.ModuleType("slangtorch"))
    sys.path.insert(0, str(root))
    import dsplat.fmcw as fmcw  # noqa: E402
    import dsplat.groundtruth as groundtruth  # noqa: E402

    out: dict[str, np.ndarray] = {}
    config = fmcw.FMCWConfig()
    side = 16
    positions = groundtruth.planar_array(side, config.lambda_m / 4, standoff=0.3)
    g = torch.Generator().manual_seed(19)
    centers = torch.tensor([0.0, 0.0, 0.3]) + torch.tensor([0.006, 0.006, 0.004]) * (
        2 * torch.rand(4, 3, generator=g) - 1)  # fmt: skip
    normals = torch.tensor([0.0, 0.0, -1.0]).expand(4, 3).clone()
    amplitudes = torch.complex(0.5 + torch.rand(4, generator=g), 0.2 * torch.randn(4, generator=g)) * 0.003
    scan = groundtruth.synthesize(positions, centers, normals, amplitudes, config)
    out["positions"], out["data"] = positions.numpy(), scan.data.numpy()
    axis = torch.linspace(-0.008, 0.008, 17)
    x, y = torch.meshgrid(axis, axis, indexing="ij")
    plane = torch.stack([x.flatten(), y.flatten(), torch.full_like(x.flatten(), 0.3)], -1)
    volume = torch.cat([plane[::3] + torch.tensor([0.0, 0.0, dz]) for dz in (-0.004, -0.001, 0.002, 0.005)])
    for name, points, padding in (("plane", plane, 2), ("volume", volume, 3)):
        strength = fmcw.migration(scan, points, (side, side), padding=padding)
        out[f"{name}_points"], out[f"{name}_strength"] = points.numpy(), strength.numpy()
        out[f"{name}_padding"] = np.array([padding])
    np.savez_compressed(HERE / "reference_migration.npz", **out)
    print("wrote", HERE / "reference_migration.npz")


if __name__ == "__main__":
    # --scene / --migration regenerate only reference_scene.npz / reference_migration.npz
    flags = {"--scene", "--migration"}
    args = [a for a in sys.argv[1:] if a not in flags]
    root = reference_root(args)
    chosen = flags & set(sys.argv)
    if not chosen:
        main(root)
    if not chosen or "--scene" in chosen:
        scene_cases(root)
    if not chosen or "--migration" in chosen:
        migration_cases(root)
