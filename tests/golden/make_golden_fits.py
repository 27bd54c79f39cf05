"""Run the reference's own DSFW solver on small scenes and record its objective histories.

Run here, where the reference checkout exists:

    python tests/golden/make_golden_fits.py /path/to/Dirichlet-Splatting   (or set DSPLAT_REFERENCE)

The reference's Python solver (dsplat/dsfw.py, varpro.py, replacement.py,
refinement.py, certificate.py, parameters.py, fmcw.py, spectral.py) runs unmodified;
only its kernel-binding modules (dsplat/kernels/*.py, which launch Slang through
slangtorch and need a GPU) are replaced, before import, by float64 CPU restatements
from this repository's oracle/, and the products it would compute on the GPU keep
their GPU arithmetic: the cuBLAS SSYRK of the normal equations accumulates in float32,
and the Gauss-Newton probe signs are the draws of a CUDA generator (recorded by
record_cuda_signs.py into cuda_rademacher.npz), not of the CPU generator. Two more runs
perturb every model-kernel output by relative noise of 1e-6 and 1e-5 and record how far
the trajectory moves ("spread"). The records go to tests/golden/reference_fits.json;
tests/test_fits_gpu.py runs the same scenes through the GB300 package on CUDA.
"""

from __future__ import annotations

import json
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


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


# Relative perturbation of every model-kernel output (0: exact oracle values). Runs with
# a small perturbation show how far the reference's own trajectory moves under the
# rounding noise that float32 kernels bring; the tests allow that spread.
NOISE = {"scale": 0.0, "generator": torch.Generator().manual_seed(0)}


def _perturb(value):
    if isinstance(value, tuple):
        return tuple(_perturb(v) for v in value)
    if not isinstance(value, torch.Tensor) or NOISE["scale"] == 0.0 or not value.is_floating_point() and not value.is_complex():
        return value
    g = NOISE["generator"]
    noise = torch.randn(value.shape, generator=g, dtype=torch.float64)
    if value.is_complex():
        noise = torch.complex(noise, torch.randn(value.shape, generator=g, dtype=torch.float64))
    return (value.to(noise.dtype) * (1 + NOISE["scale"] * noise)).to(value.dtype)


def _perturbed(fn):
    def wrapper(*args, **kwargs):
        return _perturb(fn(*args, **kwargs))

    wrapper.__name__ = fn.__name__
    return wrapper


def _shim_modules():
    """Kernel-binding modules with the reference's signatures, computed by the oracle."""
    sys.path.insert(0, str(REPO))
    from oracle import fmcw as ofmcw
    from oracle import search as osearch
    from oracle import spectral as ospectral

    c64, f32 = torch.complex64, torch.float32

    surfel = types.ModuleType("dsplat.kernels.surfel")

    def render(config, positions, centers, normals, weights, fresnel_n):
        return ofmcw.render(config, positions, centers.detach(), normals.detach(), weights.detach(),
                            fresnel_n).to(c64)  # fmt: skip

    def jvp(config, positions, centers, normals, weights, dc, dn, dw, fresnel_n):
        return ofmcw.jvp(config, positions, centers, normals, weights, dc, dn, dw, fresnel_n).to(c64)

    def vjp(config, positions, centers, normals, weights, upstream, fresnel_n):
        gc, gn, gw = ofmcw.vjp(config, positions, centers, normals, weights, upstream, fresnel_n)
        return gc.to(f32), gn.to(f32), gw.to(c64)

    def design(config, positions, centers, normals, areas, fresnel_n, real):
        out = ofmcw.design(config, positions, centers, normals, areas, fresnel_n, real)
        return out.to(f32) if real else out.to(c64)

    def jacobian(config, positions, centers, normals, fresnel_n):
        pos, cen, nrm = positions.double(), centers.double(), normals.double()
        cols = ofmcw.columns(pos, cen, nrm, config, fresnel_n)
        parts = []
        for key in ("centers", "normals"):
            for axis in range(3):
                tc, tn = torch.zeros_like(cen), torch.zeros_like(nrm)
                (tc if key == "centers" else tn)[:, axis] = 1.0
                _, d = torch.func.jvp(lambda c, n: ofmcw.columns(pos, c, n, config, fresnel_n), (cen, nrm),
                                      (tc, tn))  # fmt: skip
                parts.append(d)
        jac = torch.stack(parts, -1).to(c64)
        return cols.to(c64), jac[..., :3], jac[..., 3:]

    def correlate(config, positions, centers, normals, residual, fresnel_n):
        corr, norm = ofmcw.correlate(config, positions, centers, normals, residual, fresnel_n)
        return corr.to(c64), norm.to(f32)

    def correlate_gradient(config, positions, centers, normals, residual, fresnel_n, include_normals):
        out = ofmcw.correlate_gradient(config, positions, centers, normals, residual, fresnel_n, include_normals)
        return out[0].to(c64), out[1].to(f32), out[2].to(c64), out[3].to(f32)

    def correlate_orientations(config, positions, centers, normals, bank, residual, fresnel_n, table=None):
        tab = None if table is None else (table.correlation, table.norm, table.oversample)
        corr, norm = ofmcw.correlate_orientations(config, positions, centers, normals, bank, residual,
                                                  fresnel_n, tab)  # fmt: skip
        return corr.to(c64), norm.to(f32)

    for fn in (render, jvp, vjp, design, jacobian, correlate, correlate_gradient, correlate_orientations):
        setattr(surfel, fn.__name__, fn)

    spectral = types.ModuleType("dsplat.kernels.spectral")
    spectral.design = lambda grid, centers, bins, derivatives=False: (
        tuple(x.to(c64) for x in ospectral.design(grid, centers, bins)) if derivatives
        else ospectral.design(grid, centers, bins)[0].to(c64))  # fmt: skip
    spectral.render = lambda grid, centers, coefficients, bins: ospectral.render(grid, centers, coefficients,
                                                                                 bins).to(c64)  # fmt: skip
    spectral.jvp = lambda grid, centers, b, dc, db, bins: ospectral.jvp(grid, centers, b, dc, db, bins).to(c64)

    def spectral_vjp(grid, centers, coefficients, upstream, bins):
        gc, gb = ospectral.vjp(grid, centers, coefficients, upstream, bins)
        return gc.to(f32), gb.to(c64)

    spectral.vjp = spectral_vjp

    for module in (surfel, spectral):
        for name in [n for n in vars(module) if not n.startswith("_")]:
            if callable(getattr(module, name)):
                setattr(module, name, _perturbed(getattr(module, name)))

    search = types.ModuleType("dsplat.kernels.search")
    search.range_gate = osearch.range_gate
    search.peaks = lambda scores, centers, count, separation: osearch.peaks(scores, centers, count, separation)
    search.direction = lambda inverse, gradient, normals, mask, radius: osearch.direction(
        inverse, gradient, normals, mask, radius).to(f32)
    search.trial = lambda centers, normals, direction, controls, fraction: tuple(
        x.to(f32) for x in osearch.trial(centers, normals, direction, controls, fraction))

    reduce = types.ModuleType("dsplat.kernels.reduce")
    reduce.energy = lambda value, reference: osearch.energy(value, reference)

    response = types.ModuleType("dsplat.kernels.response")
    response.range_response = lambda config, low, high, count, device: ofmcw.range_response(config, low, high,
                                                                                           count)  # fmt: skip

    cublas = types.ModuleType("dsplat.kernels.cublas")

    def syrk(rows, out):
        # cublasSsyrk_v2 accumulates in float32; so does this product (float32 CPU GEMM).
        out += torch.triu(rows.float().T @ rows.float()).to(out.dtype)

    cublas.syrk = syrk
    return {"surfel": surfel, "spectral": spectral, "search": search, "reduce": reduce,
            "response": response, "cublas": cublas}  # fmt: skip


class _RecordedGenerator:
    """A CUDA generator stand-in whose randint draws come from cuda_rademacher.npz."""

    def __init__(self, device=None):
        self.seed, self.calls = None, 0

    def manual_seed(self, seed):
        self.seed, self.calls = int(seed), 0
        return self


class _TorchWithCudaDraws(types.ModuleType):
    """torch for the reference's refinement module, except Generator and randint."""

    def __init__(self, draws):
        super().__init__("torch")
        self._draws = draws
        self.Generator = _RecordedGenerator

    def __getattr__(self, name):
        return getattr(torch, name)

    def randint(self, low, high, size, *, device=None, generator=None, **kwargs):
        if not isinstance(generator, _RecordedGenerator):
            return torch.randint(low, high, size, device=device, generator=generator, **kwargs)
        assert (low, high) == (0, 2) and size[-1] == 2, (low, high, size)
        count = int(np.prod(size))
        bits = np.unpackbits(self._draws[f"s{generator.seed}_{size[0]}x{size[1]}"])
        draw = bits[generator.calls * count : (generator.calls + 1) * count]
        assert len(draw) == count, "more recorded draws needed"
        generator.calls += 1
        return torch.as_tensor(draw.reshape(size), dtype=torch.int64, device=device)


def import_reference(root: Path):
    sys.modules.setdefault("slangtorch", types.ModuleType("slangtorch"))
    # The shims must be in place before the reference package imports its bindings.
    for name, module in _shim_modules().items():
        sys.modules[f"dsplat.kernels.{name}"] = module
    sys.path.insert(0, str(root))
    import dsplat  # noqa: E402
    import dsplat.surfel  # noqa: E402
    import dsplat.varpro  # noqa: E402

    # The reference's grid helpers default to device="cuda"; here the whole solver runs on
    # the CPU, so only those defaults change (the function bodies stay the reference's).
    import dsplat.certificate  # noqa: E402

    dsplat.certificate.candidate_grid.__defaults__ = ("cpu",)
    dsplat.certificate.fibonacci_sphere.__defaults__ = ("cpu",)
    # The Gauss-Newton probe signs are the ones a CUDA generator draws (record_cuda_signs.py).
    import dsplat.refinement  # noqa: E402

    dsplat.refinement.torch = _TorchWithCudaDraws(np.load(HERE / "cuda_rademacher.npz"))

    assert dsplat.__file__.startswith(str(root))
    assert dsplat.surfel.kernel is sys.modules["dsplat.kernels.surfel"]
    assert dsplat.varpro.syrk is sys.modules["dsplat.kernels.cublas"].syrk

    return dsplat


def aperture_grid(side=8, pitch=0.004, device="cpu"):
    t = (torch.arange(side, dtype=torch.float32) - (side - 1) / 2) * pitch
    x, y = torch.meshgrid(t, t, indexing="ij")
    return torch.stack([x.flatten(), y.flatten(), torch.zeros(side * side)], -1).to(device)


def surfels(count, seed=0, spread=0.01, device="cpu"):
    generator = torch.Generator().manual_seed(seed)
    centers = torch.tensor([0, 0, 0.3]) + spread * (2 * torch.rand(count, 3, generator=generator) - 1)
    direction = torch.tensor([0.0, 0, -1]) + 0.3 * torch.randn(count, 3, generator=generator)
    normals = torch.nn.functional.normalize(direction, dim=1)
    out = dict(centers=centers, normals=normals, areas=torch.full((count,), 1e-4))
    return {k: v.to(device) for k, v in out.items()}


def fmcw_specs(dsplat):
    return dict(
        centers=dsplat.ParameterConfig(scale=0.0005, lower=(-0.02, -0.02, 0.28), upper=(0.02, 0.02, 0.32)),
        normals=dsplat.ParameterConfig(scale=0.1, normalize=True),
        areas=dsplat.ParameterConfig(trainable=False),
    )


def _record(state):
    return {"history": [{k: float(v) for k, v in e.items()} for e in state.history],
            "centers": state.params["centers"].tolist()}  # fmt: skip


def run_scenes(dsplat, device="cpu", names=None, configure=None):
    """Every scene through the given `dsplat` package; {name: {"history", "centers"}}.

    The same code runs the reference (on the CPU, through the oracle shims) and the GB300
    package (on CUDA), so the two records differ only by the implementation. configure
    maps each scene's DSFWConfig to the one used (the GB300 package's batched mode).
    """
    results = {}
    wanted = (lambda name: True) if names is None else (lambda name: name in names)
    setup = configure or (lambda cfg: cfg)

    # FMCW: merged replacement from a displaced start, screened joint Gauss-Newton.
    config = dsplat.FMCWConfig()
    positions = aperture_grid(device=device)
    truth = surfels(5, device=device)
    coefficients = torch.linspace(0.5, 1.5, 5).to(device)
    empty = dsplat.Scan(torch.zeros((64, config.num_range_bins), dtype=torch.complex64, device=device),
                        positions, config)  # fmt: skip
    data = dsplat.FMCWModel(empty).render(truth, coefficients)
    model = dsplat.FMCWModel(dsplat.Scan(data, positions, config))
    for name, cfg in {
        "fmcw_merged_joint": dsplat.DSFWConfig(batch=5, lm_gain_ratio=0, joint_apertures=16, screen_apertures=16),
        "fmcw_merged_dense": dsplat.DSFWConfig(batch=5, lm_gain_ratio=0, lm_solver="dense", lm_rows=2048,
                                               screen_apertures=0),
    }.items():  # fmt: skip
        if not wanted(name):
            continue
        cfg = setup(cfg)
        state = dsplat.initialize(model, data, surfels(5, seed=9, device=device), cfg, candidates=truth,
                                  parameters=fmcw_specs(dsplat))  # fmt: skip
        for _ in range(4):
            state = dsplat.step(state, cfg)
        results[name] = _record(state)

    # FMCW: the pool is the truth displaced by a few tenths of a millimetre, so the fit has
    # to move every surfel with the joint Gauss-Newton step.
    if wanted("fmcw_nearby_joint"):
        generator = torch.Generator().manual_seed(21)
        cpu_truth = surfels(5)
        nearby = {"centers": cpu_truth["centers"] + 3e-4 * torch.randn(5, 3, generator=generator),
                  "normals": torch.nn.functional.normalize(
                      cpu_truth["normals"] + 0.05 * torch.randn(5, 3, generator=generator), dim=1),
                  "areas": cpu_truth["areas"].clone()}  # fmt: skip
        nearby = {k: v.to(device) for k, v in nearby.items()}
        cfg = setup(dsplat.DSFWConfig(batch=5, lm_gain_ratio=0, joint_apertures=0, screen_apertures=0, lm_steps=2))
        state = dsplat.initialize(model, data, surfels(5, seed=9, device=device), cfg, candidates=nearby,
                                  parameters=fmcw_specs(dsplat))  # fmt: skip
        for _ in range(6):
            state = dsplat.step(state, cfg)
        results["fmcw_nearby_joint"] = _record(state)

    # FMCW: no pool at all; every step proposes candidates by the spatial search (coarse
    # grid, two finer levels, the normal bank and the continuous certificate ascent).
    if wanted("fmcw_spatial_search"):
        bounds = dict(lower=(-0.012, -0.012, 0.288), upper=(0.012, 0.012, 0.312))
        specs = fmcw_specs(dsplat)
        specs["centers"] = dsplat.ParameterConfig(scale=0.0005, **bounds)
        search = dsplat.SpatialSearchConfig(proposal_apertures=64, refine_apertures=64, normal_candidates=8,
                                            cache_peaks=32, full_peaks=8)  # fmt: skip
        cfg = setup(dsplat.DSFWConfig(batch=8, lm_gain_ratio=0, joint_apertures=0, screen_apertures=0))
        state = dsplat.initialize(model, data, surfels(5, seed=9, device=device), cfg, parameters=specs)
        for _ in range(3):
            state = dsplat.step(state, cfg, search)
        results["fmcw_spatial_search"] = _record(state)

    # Spectral: a misplaced tone recovered by utility replacement and dense LM.
    if wanted("spectral_utility_dense"):
        grid = dsplat.SpectralGrid((24, 20))
        smodel = dsplat.SpectralModel(grid)
        centers = torch.tensor([[3.3, 4.1], [12.0, 15.0], [18.4, 7.9]], device=device)
        b = torch.tensor([1 + 0.5j, -0.7 + 0.2j, 0.4 - 0.9j], device=device)
        target = smodel.render({"centers": centers}, b)
        wrong = centers.clone()
        wrong[1] = torch.tensor([20.0, 2.0], device=device)
        cfg = setup(dsplat.DSFWConfig(coefficients="complex", replacement="utility", lm_solver="dense",
                                      lm_rows=grid.size, lm_gain_ratio=0, lm_steps=3))  # fmt: skip
        specs = {"centers": dsplat.ParameterConfig(period=grid.shape, scale=0.5)}
        state = dsplat.initialize(smodel, target, {"centers": wrong}, cfg,
                                  candidates={"centers": grid.bins(device)}, parameters=specs)  # fmt: skip
        for _ in range(3):
            state = dsplat.step(state, cfg)
        results["spectral_utility_dense"] = _record(state)
    return results


def _spread(runs):
    """Per step: NMSE range and replacement counts over the runs; final-center scatter."""
    first = runs[0]
    steps = []
    for i in range(len(first["history"])):
        entries = [r["history"][i] for r in runs if i < len(r["history"])]
        steps.append({"nmse_min": min(e["nmse"] for e in entries), "nmse_max": max(e["nmse"] for e in entries),
                      "replaced": sorted({e.get("replaced", -1.0) for e in entries})})  # fmt: skip
    base = torch.tensor(first["centers"], dtype=torch.float64)
    scatter = max(float(torch.cdist(torch.tensor(r["centers"], dtype=torch.float64), base).min(1).values.max())
                  for r in runs)  # fmt: skip
    return {"steps": steps, "center_scatter_m": scatter}


def main(root: Path) -> None:
    dsplat = import_reference(root)
    results = run_scenes(dsplat, "cpu")
    perturbed = []
    for seed, scale in ((1, 1e-6), (2, 1e-5)):
        NOISE["scale"], NOISE["generator"] = scale, torch.Generator().manual_seed(seed)
        perturbed.append(run_scenes(dsplat, "cpu"))
    NOISE["scale"] = 0.0
    for name, record in results.items():
        record["spread"] = _spread([record] + [run[name] for run in perturbed])
        record["spread"]["noise"] = [1e-6, 1e-5]
    (HERE / "reference_fits.json").write_text(json.dumps(results, indent=1))
    print("wrote", HERE / "reference_fits.json")
    for name, r in results.items():
        print(name, [e["objective"] for e in r["history"]])


if __name__ == "__main__":
    main(reference_root(sys.argv[1:]))
