"""Run the reference's own DSFW solver on the full-size 2-D spectrum workload and record it.

The workload: a 256 x 256 grid of band-limited Fourier samples, 80 unit tones on the outline
of a five-point star spanning 60 % of the field (dsplat.workloads.star_tones, seed 0, 20 dB
SNR), 80 atoms started uniformly at random (seed 1), 100 steps of utility replacement over
every grid bin with three dense LM steps each (the configuration of
tests/test_fits_end_to_end_gpu.py's C2 test). Run here, where the reference checkout exists:

    python tests/golden/make_golden_c2.py /path/to/Dirichlet-Splatting [exact|noise]

The reference's Python solver runs unmodified on the CPU with its kernel bindings replaced
by the float64 oracle (make_golden_fits.import_reference). "exact" records the trajectory;
"noise" perturbs every model-kernel output by 1e-6 relative noise, to measure how far the
reference's own trajectory moves under float32-level rounding. Each run takes about twenty
minutes on eight cores; the records go to tests/golden/reference_c2_fit.json.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
STEPS = 100


def main(args):
    sys.path.insert(0, str(HERE))
    sys.path.insert(0, str(REPO))
    sys.path.insert(0, str(REPO / "dirichlet-splatting_gb300"))
    import make_golden_fits as mg

    root = mg.reference_root(args[:1])
    mode = args[1] if len(args) > 1 else "exact"
    from dsplat.workloads import star_tones

    target, truth = star_tones(device="cpu")
    # the reference package must import under the name dsplat: drop this repository's
    for key in [k for k in sys.modules if k == "dsplat" or k.startswith("dsplat.")]:
        del sys.modules[key]
    sys.path.remove(str(REPO / "dirichlet-splatting_gb300"))
    reference = mg.import_reference(root)
    if mode == "noise":
        mg.NOISE["scale"] = 1e-6
    grid = reference.SpectralGrid((256, 256))
    generator = torch.Generator().manual_seed(1)
    start = {"centers": torch.rand(80, 2, generator=generator) * 256}
    config = reference.DSFWConfig(iterations=STEPS, ridge=1e-8, coefficients="complex", replacement="utility",
                                  min_separation=0.35, lm_solver="dense", lm_steps=3, lm_rows=grid.size,
                                  lm_gain_ratio=0, screen_apertures=0, trust_radius=0.75)  # fmt: skip
    state = reference.initialize(reference.SpectralModel(grid), target, start, config,
                                 candidates={"centers": grid.bins("cpu")},
                                 parameters={"centers": reference.ParameterConfig(period=grid.shape)})  # fmt: skip
    for _ in range(STEPS):
        state = reference.step(state, config)
        print(json.dumps(state.history[-1]), flush=True)
    out = HERE / "reference_c2_fit.json"
    records = json.loads(out.read_text()) if out.exists() else {}
    records[mode] = {"history": [{k: float(v) for k, v in e.items()} for e in state.history],
                     "centers": state.params["centers"].tolist(), "truth": truth.tolist()}  # fmt: skip
    out.write_text(json.dumps(records, indent=1))


if __name__ == "__main__":
    main(sys.argv[1:])
