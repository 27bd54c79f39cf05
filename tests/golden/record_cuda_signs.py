"""Record the Rademacher sign draws that the joint Gauss-Newton system makes on a CUDA device.

The reference's joint_system (dsplat/refinement.py:160-165) draws its probe signs with
torch.Generator(device=<model device>).manual_seed(seed) and torch.randint(0, 2,
(*target.shape, 2)). On a GPU those come from CUDA's Philox stream, which the CPU
generator does not reproduce; make_golden_fits.py replays these recorded CUDA draws when
it runs the reference on the CPU, so that its Gauss-Newton probes are the ones the
reference (and this package) draw on the GPU. Run on a CUDA machine:

    python tests/golden/record_cuda_signs.py tests/golden/cuda_rademacher.npz
"""

from __future__ import annotations

import sys

import numpy as np
import torch

SEEDS = range(32)
SHAPES = ((64, 128), (16, 128))  # the golden scenes' target rows x range bins
DRAWS = 4  # per seed; the default DSFWConfig.cg_probes is 2


def main(path):
    out = {}
    for shape in SHAPES:
        for seed in SEEDS:
            generator = torch.Generator(device="cuda").manual_seed(seed)
            draws = [torch.randint(0, 2, (*shape, 2), device="cuda", generator=generator) for _ in range(DRAWS)]
            bits = torch.stack(draws).to(torch.uint8).cpu().numpy()
            out[f"s{seed}_{shape[0]}x{shape[1]}"] = np.packbits(bits.reshape(-1))
    out["meta"] = np.array([DRAWS, len(SEEDS)])
    out["torch_version"] = np.array(torch.__version__)
    np.savez_compressed(path, **out)
    print("wrote", path, "with torch", torch.__version__)


if __name__ == "__main__":
    main(sys.argv[1])
