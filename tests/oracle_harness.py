"""Run this package's DSFW solver on the CPU with its kernel bindings computed by the oracle.

Test infrastructure. The product path has no CPU fallback: every binding in
dsplat/kernels calls libdsplat_gb300.so and rejects CPU tensors. To check the solver's
host logic without a GPU, this script installs, before dsplat is imported, the same
oracle-backed binding modules that tests/golden/make_golden_fits.py gives the
reference's solver (float64 closed forms cast to the kernels' float32 / complex64, a
float32-accumulating SYRK, and the Gauss-Newton probe signs a CUDA generator draws), then
runs the scenes of make_golden_fits.run_scenes through this package in plain mode and
prints their records as one JSON line:

    python tests/oracle_harness.py [scene ...]
"""

from __future__ import annotations

import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
GOLDEN = HERE / "golden"


def _golden_module():
    spec = importlib.util.spec_from_file_location("make_golden_fits", GOLDEN / "make_golden_fits.py")
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def import_package_on_oracle():
    """This repository's dsplat with oracle-backed kernel bindings (CPU only)."""
    golden = _golden_module()
    shims = golden._shim_modules()
    full_correlate = shims["surfel"].correlate

    def correlate(config, positions, centers, normals, residual, fresnel_n, active=None):
        # active only lets the CUDA kernel skip atoms whose values the caller masks.
        return full_correlate(config, positions, centers, normals, residual, fresnel_n)

    shims["surfel"].correlate = correlate
    # the spectral model's whole-grid products, restated on the oracle's per-bin bindings
    spectral = shims["spectral"]
    spectral.render_on_grid = lambda grid, centers, b: spectral.render(grid, centers, b, grid.bins(centers.device))
    spectral.jvp_grid = lambda grid, centers, b, dc, db: spectral.jvp(grid, centers, b, dc, db,
                                                                      grid.bins(centers.device))  # fmt: skip
    spectral.vjp_grid = lambda grid, centers, b, u: spectral.vjp(grid, centers, b, u.reshape(-1),
                                                                 grid.bins(centers.device))  # fmt: skip
    for name, module in shims.items():
        sys.modules[f"dsplat.kernels.{name}"] = module
    sys.path.insert(0, str(ROOT / "dirichlet-splatting_gb300"))
    import dsplat
    import dsplat.certificate
    import dsplat.refinement

    assert dsplat.__file__.startswith(str(ROOT))
    dsplat.certificate.candidate_grid.__defaults__ = ("cpu",)
    dsplat.certificate.fibonacci_sphere.__defaults__ = ("cpu",)
    draws = np.load(GOLDEN / "cuda_rademacher.npz")
    dsplat.refinement.probe_signs = _recorded_probe_signs(draws)
    return dsplat, golden


def _recorded_probe_signs(draws):
    """probe_signs(shape, seed, device) -> a generator of the CUDA draws recorded for seed."""

    def probe_signs(shape, seed, device):
        count = int(np.prod(shape))
        bits = np.unpackbits(draws[f"s{seed}_{shape[0]}x{shape[1]}"])
        call = 0
        while True:
            draw = bits[call * count : (call + 1) * count]
            assert len(draw) == count, "more recorded draws needed"
            import torch

            yield torch.as_tensor(draw.reshape(shape), dtype=torch.int64, device=device)
            call += 1

    return probe_signs


def main(names):
    dsplat, golden = import_package_on_oracle()
    results = golden.run_scenes(dsplat, "cpu", names=set(names) if names else None)
    print(json.dumps(results))


if __name__ == "__main__":
    main(sys.argv[1:])
