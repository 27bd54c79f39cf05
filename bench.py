"""Benchmark: DSFW steps/s of the 128^2-array, 2000-surfel sphere-cap fit (batch 256).

Our arm (default): the drop-in dsplat package on libdsplat_gb300.so, mixed precision
and batched execution (split-BF16x3 tcgen05 Gram, DSFWConfig(gram="bf16x3",
batched=True)); --mode plain is the FP32 drop-in. Workload: the 128 x 128 array at
2.5 mm pitch, 2000 surfels on the front hemisphere of a 30 mm sphere at 0.35 m, scan
synthesized in float64 from the ADC signal chain, a 100-step fit from random surfels in
the box plus 5 mm with SpatialSearchConfig() and DSFWConfig(batch=256). W untimed
warm-up steps after initialize; `value` times steps W+1..W+K with the inputs resident in
HBM and nothing instrumented; `e2e` times the same steps again from the same state with
the step's inputs copied in from pinned host memory and its result copied out; a third,
instrumented pass over the same steps gives the per-kernel table and the roofline. The
fit then runs on to step 100, and the plain FP32 fit runs all 100 steps from the same
start: the speed-up compares the same step indices, and the final NMSE and median
centre-to-surface distance of the two fits are compared (within 5 %).

Reference arm (--impl reference): the float64 CPU oracle (oracle/solver.py) on the
host cores: one full-size refit (all 16 384 apertures) timed whole, and a step counted
as the refit-equivalents of Gram work that a GB300 step performs.

Prints one JSON line (rank 0).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _path in (ROOT, ROOT / "dirichlet-splatting_gb300"):
    if str(_path) not in sys.path:
        sys.path.insert(0, str(_path))

import torch  # noqa: E402

METRIC = "DSFW steps/s (128² array, 2k surfels) mixed+batched vs plain FP32; equal NMSE"
UNIT = "steps/s"
WORKLOAD = "dsfw_sphere_cap_128x128_s2000_b256"
# One config for both arms.
CONFIG = {"workload": WORKLOAD, "apertures": 16384, "range_bins": 128, "surfels": 2000, "batch": 256,
          "iterations": 100, "search": "SpatialSearchConfig()",
          "l2": "256 MiB buffer written between timed steps", "parallelism": "replicas"}  # fmt: skip


def _peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return data, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def _distributed():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not torch.distributed.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        torch.distributed.init_process_group(backend)
    return world, rank, local


def _barrier(world):
    if world > 1:
        torch.distributed.barrier()


def _max_over_ranks(value, world, device):
    if world == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")  # fmt: skip

    def __init__(self, index):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)  # fmt: skip
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        lines = [ln.strip() for ln in Path(self.file.name).read_text().splitlines() if ln.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9], strict=True):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}  # fmt: skip


def build_problem(device, seed=0):
    """Scan, initial surfels and constraints of the sphere-cap fit (all on device)."""
    from dsplat import FMCWConfig, FMCWModel, ParameterConfig
    from dsplat.groundtruth import synthesize
    from dsplat.workloads import box_of, random_start, sphere_cap

    config = FMCWConfig()
    positions, truth, reflectivity = sphere_cap(device=device, seed=seed)
    amplitudes = reflectivity * truth["areas"].sqrt()
    scan = synthesize(positions, truth["centers"], truth["normals"], amplitudes, config)
    low, high = box_of(truth["centers"], 0.005)
    start = random_start(len(truth["centers"]), low, high, float(truth["areas"][0]), seed=seed + 1,
                         device=device)  # fmt: skip
    parameters = dict(
        centers=ParameterConfig(scale=5e-4, lower=low, upper=high),
        normals=ParameterConfig(scale=0.1, normalize=True),
        areas=ParameterConfig(trainable=False),
    )
    return FMCWModel(scan=scan), scan.data, start, parameters, truth


def median_distance(params, truth, radius=0.03, depth=0.35):
    c = params["centers"].double()
    center = torch.tensor([0.0, 0.0, depth], dtype=torch.float64, device=c.device)
    return float(((c - center).norm(dim=1) - radius).abs().median())


UNEVEN_WORKLOAD = "dsfw_uneven_64_scenes_10_steps_b128"


def run_uneven(args):
    """The many-scene workload: 64 uneven FMCW scenes, 10 DSFW steps each, batch 128.

    Scenes (dsplat.workloads.uneven_scenes): array side in {32, 64, 96, 128}, 128 or 256 ADC
    samples, 200-4000 surfels on ellipsoid caps (semi-axes 15-40 mm, depth 0.30-0.45 m).
    Mixed precision and batched execution, launch shapes tuned on the largest scene. The
    rounds (one step of every scene) are timed with CUDA events; value = all scenes' steps
    per second. The batch's data NMSE comes from one persistent render of every scene.
    """
    import __graft_entry__

    __graft_entry__.build()
    from dsplat import DSFWConfig, SpatialSearchConfig, autotune, initialize, step
    from dsplat.kernels import surfel as kernel
    from dsplat.scenes import batch_nmse, problems_from_scenes, render_states
    from dsplat.workloads import uneven_scenes

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    config = DSFWConfig(iterations=args.rounds, batch=128, gram="bf16x3", batched=True)
    search = SpatialSearchConfig()
    problems = problems_from_scenes(uneven_scenes(args.scenes, seed=0, device=device))
    states = [initialize(p.model, p.target, p.start, config, parameters=p.parameters) for p in problems]
    if not args.no_autotune:
        largest = max(range(len(states)), key=lambda i: states[i].model.size * len(states[i].coefficients))
        chirp, positions = states[largest].model.sensor
        basis = states[largest].model.block_basis(slice(0, min(2048, len(positions)) * chirp.num_range_bins))
        autotune.tune_workload(chirp, positions, states[largest].params,
                               states[largest].target - states[largest].prediction, basis)  # fmt: skip
    start_nmse = batch_nmse(states)
    # one batched render of every scene against one launch per scene
    torch.cuda.synchronize(device)
    per_scene = autotune.time_cuda(lambda: [kernel.render(*s) for s in _render_batch(states)], repeats=3)
    batched = autotune.time_cuda(lambda: render_states(states), repeats=3)
    rounds_ms = []
    for _ in range(config.iterations):
        begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        begin.record()
        states = [step(state, config, search) for state in states]
        end.record()
        end.synchronize()
        rounds_ms.append(begin.elapsed_time(end))
    final_nmse = batch_nmse(states)
    total_s = sum(rounds_ms) / 1e3
    steps = len(states) * config.iterations
    result = {
        "metric": "DSFW steps/s over 64 uneven scenes (10 steps each, batch 128), mixed+batched",
        "value": round(steps / total_s, 4), "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 0,
        "ms_per_step": round(total_s * 1e3 / steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+bf16x3", "data": "synthetic (float64 ADC synthesis of seeded ellipsoid caps)",
        "config": {"workload": UNEVEN_WORKLOAD, "scenes": len(states), "rounds": config.iterations, "batch": 128},
        "round_ms": [round(t, 1) for t in rounds_ms],
        "batch_render_ms": {"one_persistent_launch": round(batched, 3), "one_launch_per_scene": round(per_scene, 3)},
        "batch_nmse": {"start_mean": sum(start_nmse) / len(start_nmse), "final_mean": sum(final_nmse) / len(final_nmse),
                       "final_max": max(final_nmse), "improved_scenes": sum(f < s for f, s in
                                                                            zip(final_nmse, start_nmse))},
    }  # fmt: skip
    print(json.dumps(result), flush=True)


def _render_batch(states):
    batch = []
    for state in states:
        config, positions = state.model.sensor
        weights = state.coefficients.to(torch.complex64) * state.params["areas"].sqrt()
        batch.append((config, positions, state.params["centers"], state.params["normals"], weights,
                      state.model.fresnel_n))  # fmt: skip
    return batch


def run_accuracy(args):
    """Final NMSE and centre-to-surface distance of both arms over several scenes.

    One fit is a chaotic sequence of discrete decisions (which candidates enter, which
    slides pass), so two arithmetics that agree to rounding still reach different final
    states. This mode runs the 100-step fit of the plain FP32 arm and of the mixed+batched
    arm on args.accuracy seeded scenes (sphere cap and start drawn from the seed) and
    reports each pair and the means, to compare the arms' spread with their difference.
    """
    import __graft_entry__

    __graft_entry__.build()
    from dsplat import DSFWConfig, SpatialSearchConfig, initialize, step

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    search = SpatialSearchConfig()
    arms = {"plain_fp32": DSFWConfig(iterations=args.iterations, batch=256),
            "mixed_batched": DSFWConfig(iterations=args.iterations, batch=256, gram="bf16x3", batched=True)}
    runs = []
    for seed in range(args.accuracy):
        model, target, start, parameters, truth = build_problem(device, seed=seed)
        record = {"seed": seed}
        for name, config in arms.items():
            state = initialize(model, target, start, config, parameters=parameters)
            for _ in range(config.iterations):
                state = step(state, config, search)
            record[name] = _fit_figures(state, truth)
        runs.append(record)
        print(json.dumps(record), flush=True)
    means = {name: {key: statistics.fmean(r[name][key] for r in runs)
                    for key in ("nmse", "median_center_to_surface_m")} for name in arms}  # fmt: skip
    gaps = {key: _gap(means["mixed_batched"][key], means["plain_fp32"][key]) for key in means["plain_fp32"]}
    print(json.dumps({"accuracy": runs, "means": means, "relative_gap_of_means": gaps}), flush=True)


def _timed_steps(state, config, search, count, flush, device):
    """Run count steps, each timed with CUDA events on the launching stream after an L2 flush."""
    from dsplat import step

    pairs = []
    for _ in range(count):
        flush.view(torch.float32).fill_(1.0)  # 256 MiB written by one fill kernel: L2 flushed
        begin = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        begin.record()
        state = step(state, config, search)
        end.record()
        pairs.append((begin, end))
    torch.cuda.synchronize(device)
    return state, [b.elapsed_time(e) for b, e in pairs]


def _fit_figures(state, truth):
    entry = state.history[-1]
    return {"iteration": entry["iteration"], "nmse": entry["nmse"],
            "median_center_to_surface_m": median_distance(state.params, truth)}  # fmt: skip


def _gap(mine, theirs):
    return abs(mine - theirs) / max(abs(theirs), 1e-300)


def run_ours(args, world, rank, local):
    """Mixed+batched arm (default) or plain arm; every arm times the same step indices.

    Order of work, all from one initialize():
      0. one discarded step of each arm from its own initialize() (process warm-up: lazy
         library loads and the first CUDA-graph captures, which would otherwise land in
         step 1 of whichever arm runs first);
      1. steps 1..W untimed (warm-up), state S_W kept;
      2. value: steps W+1..W+K from S_W, device-resident, nothing instrumented;
      3. e2e: steps W+1..W+K again from S_W (the step is a pure function of the state and
         the seeds), each step's inputs copied in from pinned host memory and its result out;
      4. kernel table: steps W+1..W+K again from S_W with per-entry-point CUDA events and
         stage ranges on (untimed for value; gives kernel_ms, stage_ms and the roofline);
      5. the fit continued from step W+K to the configured 100 steps (each step timed), for
         the final NMSE / centre-to-surface distance and the average rate over steps 1..100;
      6. with --mode mixed: the plain FP32 fit from the same start, 100 steps, each timed;
         its steps W+1..W+K are the denominator of speedup_vs_plain_fp32.
    """
    import __graft_entry__

    __graft_entry__.build()
    from dataclasses import replace

    from dsplat import DSFWConfig, SpatialSearchConfig, initialize, step, tracing
    from dsplat.kernels import _lib

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    lib = _lib.library()
    model, target, start, parameters, truth = build_problem(device)
    mixed = args.mode == "mixed"
    config = DSFWConfig(iterations=args.iterations, batch=256, gram="bf16x3" if mixed else "fp32", batched=mixed)
    search = SpatialSearchConfig()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)  # 256 MiB > L2
    _lib.TIMERS = None
    tracing.disable()

    # Process warm-up, untimed and discarded: one step of each arm from the start loads the
    # lazily loaded libraries (cuSOLVER, cuFFT, cuBLAS handles) and captures the CUDA graphs
    # that later searches of the same shapes replay, so no timed step of either arm pays a
    # one-time cost. The fits below start again from initialize().
    for warm_config in (config, DSFWConfig(iterations=args.iterations, batch=256)):
        step(initialize(model, target, start, warm_config, parameters=parameters), warm_config, search)
    torch.cuda.synchronize(device)
    init_begin = time.perf_counter()
    state = initialize(model, target, start, config, parameters=parameters)
    torch.cuda.synchronize(device)
    init_s = time.perf_counter() - init_begin
    tuned = None
    if not args.no_autotune:
        # launch shapes from the autotuner, chosen on this workload's shapes (untimed)
        from dsplat import autotune

        chirp, positions = state.model.sensor
        basis = state.model.block_basis(slice(0, min(2048, len(positions)) * chirp.num_range_bins))
        chosen = autotune.tune_workload(chirp, positions, state.params, state.target - state.prediction, basis)
        tuned = {family: value for family, (value, _) in chosen.items()}
    state, warm_ms = _timed_steps(state, config, search, args.warmup, flush, device)
    saved = state  # DSFWState is immutable: steps build new states and never write tensors in place

    # 2. value
    launches0 = lib.dsg_launch_count() + _lib.REPLAYED_LAUNCHES
    with ClockSampler(local) as clocks:
        _barrier(world)
        torch.cuda.synchronize(device)
        torch.cuda.nvtx.range_push("timed_steps")  # ncu --nvtx --nvtx-include "timed_steps/"
        state, step_ms = _timed_steps(saved, config, search, args.steps, flush, device)
        torch.cuda.nvtx.range_pop()
        # One more flush-sized fill after the last timed step: in a kernel launch list the
        # timed steps lie between the first and the last of these fills.
        flush.view(torch.float32).fill_(2.0)
        torch.cuda.synchronize(device)
        _barrier(world)
    launches = lib.dsg_launch_count() + _lib.REPLAYED_LAUNCHES - launches0
    total_s = _max_over_ranks(sum(step_ms) / 1e3, world, device)
    value = world * args.steps / total_s
    after_value = state

    # 3. e2e over the same steps
    host_target = target.cpu().pin_memory()
    e2e_times, h2d, d2h = [], 0, 0
    state = saved
    _barrier(world)
    for _ in range(args.steps):
        host_params = {k: v.cpu().pin_memory() for k, v in state.params.items()}
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        dev_target = host_target.to(device, non_blocking=True)
        dev_params = {k: v.to(device, non_blocking=True) for k, v in host_params.items()}
        h2d = host_target.numel() * 8 + sum(v.numel() * 4 for v in host_params.values())
        state = replace(state, target=dev_target, params=dev_params)
        state = step(state, config, search)
        out_params = {k: v.to("cpu") for k, v in state.params.items()}
        out_coef = state.coefficients.to("cpu")
        d2h = sum(v.numel() * 4 for v in out_params.values()) + out_coef.numel() * 4 + 8
        torch.cuda.synchronize(device)
        e2e_times.append(time.perf_counter() - t0)
    del out_params, out_coef
    e2e_total = _max_over_ranks(sum(e2e_times), world, device)
    e2e_value = world * args.steps / e2e_total
    e2e_same = abs(state.objective - after_value.objective) <= 1e-6 * abs(after_value.objective)

    # 4. kernel table (instrumented, untimed for value)
    tracing.enable()
    _lib.TIMERS, _lib.WORK = {}, {}
    state = saved
    for _ in range(args.steps):
        state = step(state, config, search)
    torch.cuda.synchronize(device)
    timers, _lib.TIMERS = _lib.TIMERS, None
    work, _lib.WORK = dict(_lib.WORK), {}
    stages = tracing.report()
    tracing.disable()
    totals = {name: sum(b.elapsed_time(e) for b, e in pairs) for name, pairs in timers.items()}
    roofline = _roofline(totals, timers, work, args)

    # 5. the rest of the fit
    state, rest_ms = _timed_steps(after_value, config, search, max(0, config.iterations - args.warmup - args.steps),
                                  flush, device)  # fmt: skip
    fit_ms = warm_ms + step_ms + rest_ms
    result = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+bf16x3" if mixed else "f32",
        "data": "synthetic (float64 ADC synthesis of a seeded sphere-cap scene)",
        "config": CONFIG,
        "mode": args.mode,
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "same_steps_as_value": True,
                "same_final_objective_as_value": bool(e2e_same)},  # fmt: skip
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "roofline": roofline,
        "tensor_roofline": None if roofline and roofline["bound"] == "tensor" else _tensor_roofline(totals, timers, work),
        "kernel_ms": {k: round(v, 3) for k, v in sorted(totals.items(), key=lambda kv: -kv[1])},
        "stage_ms": stages,
        "autotuned_launch_shapes": tuned,
        "timing": {"value_steps": f"{args.warmup + 1}..{args.warmup + args.steps}", "instrumented": False,
                   "kernel_ms_from": "a separate instrumented pass over the same steps",
                   "initialize_s": round(init_s, 3)},  # fmt: skip
        "fit_after_timed_steps": _fit_figures(after_value, truth),
        "fit_final": _fit_figures(state, truth),
        "steps_1_to_final": {"steps": len(fit_ms), "value": round(len(fit_ms) / (sum(fit_ms) / 1e3), 4),
                             "ms_per_step": round(sum(fit_ms) / len(fit_ms), 3),
                             "step_ms": [round(t, 1) for t in fit_ms],
                             "replaced": [e.get("replaced") for e in state.history[1:]],
                             "lm_accepted": [e.get("lm_accepted") for e in state.history[1:]]},  # fmt: skip
    }
    mixed_gram = work.get("dsg_gram_bf16x3")
    if mixed and not args.no_plain:
        plain = DSFWConfig(iterations=args.iterations, batch=256)
        other = initialize(model, target, start, plain, parameters=parameters)
        other, plain_ms = _timed_steps(other, plain, search, plain.iterations, flush, device)
        window = plain_ms[args.warmup : args.warmup + args.steps]
        plain_s = _max_over_ranks(sum(window) / 1e3, world, device)
        plain_value = world * args.steps / plain_s
        final = _fit_figures(other, truth)
        mine = result["fit_final"]
        keys = ("nmse", "median_center_to_surface_m")
        # signed: (mixed - plain) / plain; a negative gap is a better mixed fit
        gaps = {key: (mine[key] - final[key]) / max(abs(final[key]), 1e-300) for key in keys}
        within = all(gap <= 0.05 for gap in gaps.values())
        result["plain_fp32"] = {"value": round(plain_value, 4), "ms_per_step": round(plain_s * 1e3 / args.steps, 3),
                                "steps_1_to_final": {"steps": len(plain_ms),
                                                     "value": round(len(plain_ms) / (sum(plain_ms) / 1e3), 4),
                                                     "step_ms": [round(t, 1) for t in plain_ms]},
                                "fit_final": final}  # fmt: skip
        result["speedup_vs_plain_fp32"] = round(value / plain_value, 3)
        result["speedup_vs_plain_fp32_steps_1_to_final"] = round(
            result["steps_1_to_final"]["value"] / result["plain_fp32"]["steps_1_to_final"]["value"], 3)
        result["accuracy_vs_plain"] = {"signed_relative_gap": {k: round(v, 4) for k, v in gaps.items()},
                                       "not_worse_than_plain_by_5pct": bool(within),
                                       "meets_metric": bool(within),
                                       "note": "one seed; the fit is chaotic, see --accuracy for the seed study"}  # fmt: skip
    if mixed_gram:
        from dsplat.varpro import projected_rows, row_chunk

        full = projected_rows(saved.model, row_chunk(saved.model, 2000, config)) * 2000 * 2001
        result["refit_equivalents_per_step"] = round(mixed_gram / args.steps / full, 3)
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.cpu_threads, refits_per_step=result.get("refit_equivalents_per_step"))
    return result


TENSOR_KERNELS = ("dsg_gram_bf16x3", "dsg_design_project_bf16x3")
# DRAM bytes (read + write) per logical flop, from ncu captures of smaller launches of the
# same kernels, scaled to each launch by its work (see profiles/).
TRAFFIC_PER_FLOP = {
    # profiles/design_project_bf16x3_2048ap_1000s.md: 327.3 MB of DRAM traffic for 48.2 GFLOP
    "dsg_design_project_bf16x3": 327.3e6 / 48.2e9,
    # profiles/gram_bf16x3_200k_rows_1000.md: 889.7 MB of DRAM traffic for 200.2 GFLOP
    "dsg_gram_bf16x3": 889.7e6 / 200.2e9,
}


def _roofline(totals, timers, work, args):
    peaks, source = _peaks()
    if not totals:
        return None
    name = max(totals, key=totals.get)
    launches = len(timers[name])
    avg_ms = totals[name] / launches
    if name in TENSOR_KERNELS:
        # Logical FP32 work (the Gram: R S (S + 1) for a full symmetric product; the fused
        # projection: 4 K rank2 per aperture-surfel pair) over the launches' measured time,
        # against the sustained bf16 tensor peak / 3 (three bf16 products per logical
        # multiply-add in split-BF16x3).
        flops = work.get(name)
        achieved = flops / (totals[name] * 1e-3) / 1e12 if flops else None
        peak = peaks["bf16_tflops_sustained"] / 3
        per_launch = flops / launches if flops else None
        traffic = TRAFFIC_PER_FLOP.get(name)
        return {"kernel": name, "bound": "tensor", "achieved": achieved and round(achieved, 2),
                "peak": round(peak, 2), "unit": "TFLOP/s",
                "frac": achieved and round(achieved / peak, 4),
                "traffic": traffic and per_launch and round(traffic * per_launch),
                "peak_source": f"{source} bf16_tflops_sustained / 3", "launches": launches,
                "avg_ms": round(avg_ms, 4)}  # fmt: skip
    flops = work.get(name)
    if flops:
        # FP32-issue-bound kernels (splat forward / JVP / VJP, certificate correlations, the
        # normal bank): FP32 flops per pair-bin or pair-normal (the work-unit counts) over the
        # launches' time, against the nominal FP32 rate at the measured maximum SM clock
        # (152 SMs x 128 lanes x 2 flops); the measured-peaks file has no FP32 figure.
        mhz = peaks.get("sm_max_mhz", 2070.0)
        peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
        achieved = flops / (totals[name] * 1e-3) / 1e12
        return {"kernel": name, "bound": "fp32", "achieved": round(achieved, 2), "peak": round(peak, 1),
                "unit": "TFLOP/s", "frac": round(achieved / peak, 4), "traffic": None,
                "peak_source": f"nominal FP32 at {source} sm_max_mhz", "launches": launches,
                "avg_ms": round(avg_ms, 4)}  # fmt: skip
    return {"kernel": name, "bound": "hbm", "achieved": None, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": None, "traffic": None, "launches": launches, "avg_ms": round(avg_ms, 4)}  # fmt: skip


def _tensor_roofline(totals, timers, work):
    """The same figures for the tensor-core kernel with the largest time, when it is not the top."""
    tensor = [k for k in TENSOR_KERNELS if k in totals]
    if not tensor:
        return None
    name = max(tensor, key=totals.get)
    return _roofline({name: totals[name]}, {name: timers[name]}, work, None)


# Full-refit equivalents of one DSFW step of the mixed arm: the tcgen05 Gram work of a step
# (normal equations, pooled cross-Gram) divided by the Gram work of one full-size refit
# (R S (S + 1) logical flops, R the projected rows of all 16 384 apertures at S = 2000).
# Counted by `python bench.py` on a GB300 (key "refit_equivalents_per_step" of its line);
# the reference arm, which runs no GPU code, uses this committed count.
REFIT_EQUIVALENTS_PER_STEP = 0.442  # steps 6..25 of the GB300 bench run (value 8.03 steps/s)


def _cpu_scene(stride):
    """Sphere-cap apertures (every stride-th per axis), truth, start and box on the CPU."""
    from dsplat.workloads import box_of, random_start, sphere_cap

    positions, truth, reflectivity = sphere_cap(device="cpu")
    grid = positions.reshape(128, 128, 3)[::stride, ::stride].reshape(-1, 3).contiguous()
    low, high = box_of(truth["centers"], 0.005)
    params = random_start(2000, low, high, float(truth["areas"][0]), seed=1, device="cpu")
    return grid, truth, reflectivity, params, low, high


def cpu_baseline(threads=None, sample_stride=4, refits_per_step=None):
    """Float64 oracle refit on a 1/stride^2 aperture sample (a bounded sample), scaled to a step."""
    from dsplat import FMCWConfig

    from oracle import fmcw as ofmcw
    from oracle import solver as osolver

    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    config = FMCWConfig()
    grid, truth, reflectivity, params, low, high = _cpu_scene(sample_stride)
    amplitudes = reflectivity * truth["areas"].sqrt()
    target = ofmcw.synthesize(grid, truth["centers"], truth["normals"], amplitudes, config)
    adjoint = osolver.row_basis(config, grid, low, high)
    sample_s = osolver.timed_refit(config, grid, params, target, adjoint)
    solve_s = osolver.timed_solve(2000)
    scale = 16384 / len(grid)
    refit_s = sample_s * scale + solve_s
    count = refits_per_step or REFIT_EQUIVALENTS_PER_STEP
    return {"value": 1.0 / (count * refit_s), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"float64 VarPro refit (closed-form columns, row-basis projection, normal equations, "
                       f"Cholesky, rendered objective) on every {sample_stride}th aperture per axis "
                       f"({len(grid)} of 16384) x 2000 surfels: {sample_s:.2f} s, scaled x{scale:.0f} "
                       f"+ {solve_s:.3f} s full-size solve = {refit_s:.1f} s per full refit; a DSFW step counted "
                       f"as {count:.2f} full refits (its Gram work, counted on the GPU run); the spatial search, "
                       f"eliminations and slides are not included, so this is an upper bound on the CPU step rate")}


def full_refit_baseline(threads=None):
    """The float64 oracle restatement on the host cores: one full-size refit, timed whole.

    No sampling and no scaling: all 16 384 apertures x 2000 surfels (closed-form columns,
    row-basis projection, normal equations, Cholesky, rendered objective), chunked over
    apertures. The target is a seeded complex Gaussian scan of the workload's shape (the
    refit's cost does not depend on its values; synthesizing the true scan on the CPU would
    cost as much again). Steps/s = 1 / (refit-equivalents per step x the measured refit time).
    """
    from dsplat import FMCWConfig

    from oracle import solver as osolver

    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    wall0 = time.perf_counter()
    config = FMCWConfig()
    grid, _, _, params, low, high = _cpu_scene(1)
    generator = torch.Generator().manual_seed(0)
    shape = (len(grid), config.num_range_bins)
    target = torch.complex(torch.randn(shape, generator=generator, dtype=torch.float64),
                           torch.randn(shape, generator=generator, dtype=torch.float64)) * 1e-4  # fmt: skip
    adjoint = osolver.row_basis(config, grid, low, high)
    refit_s = osolver.timed_refit(config, grid, params, target, adjoint)
    value = 1.0 / (REFIT_EQUIVALENTS_PER_STEP * refit_s)
    sample = (f"one full-size float64 VarPro refit, 16384 apertures x 2000 surfels x 128 bins, measured whole: "
              f"{refit_s:.1f} s on {threads} threads; a DSFW step counted as {REFIT_EQUIVALENTS_PER_STEP:.2f} full "
              f"refits (the Gram work of a mixed-arm step counted on a GB300); search, eliminations and slides "
              f"excluded, so an upper bound on the CPU step rate")  # fmt: skip
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "refit_s": round(refit_s, 3), "refits_per_step": REFIT_EQUIVALENTS_PER_STEP,
            "wall_s": round(time.perf_counter() - wall0, 2)}  # fmt: skip


def run_reference(args, world, rank):
    """Rank 0 prints the reference arm's line; the other ranks exit without work."""
    if rank != 0:
        return None
    base = full_refit_baseline(args.cpu_threads)
    value = base["value"]
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference", "config": CONFIG, "cpu_baseline": base,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Slang kernels need slangtorch, which is not installed (no network); the "
                "reference arm is the float64 oracle restatement of the path on the host cores",
    }  # fmt: skip


def _event_time(fn, iterations, warmup, flush):
    """Average milliseconds of fn() over iterations, CUDA events, L2 flushed before each."""
    for _ in range(warmup):
        fn()
    total = 0.0
    for _ in range(iterations):
        flush.zero_()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        fn()
        end.record()
        torch.cuda.synchronize()
        total += start.elapsed_time(end)
    return total / iterations


def _time_elimination(rows, support, generator, device, iterations, warmup, flush):
    """Backward elimination at the pooled size of the fit (support + 256 candidates, 256
    removals, factor form, one launch per removal), appended to rows."""
    from dsplat.kernels import search

    pooled = support + 256
    x = torch.randn(pooled + 344, pooled, generator=generator, dtype=torch.float64).to(device)
    xq = x.mT @ torch.randn(pooled + 344, generator=generator, dtype=torch.float64).to(device)
    xfac = search.triangular_inverse(torch.linalg.cholesky(x.mT @ x))
    ms = _event_time(lambda: search.backward_elimination_factor(xfac, xq, 256), iterations, warmup, flush)
    rows.append({"kernel": f"dsg_backward_elimination_factor ({pooled} unknowns, 256 removals)", "ms": round(ms, 3)})


def run_kernels(args):
    """Per-kernel roofline table on the sphere-cap geometry (the workload of the DSFW bench).

    full: 128^2 apertures x 2000 surfels (C3 sizes); medium: 64^2 x 1000 (inputs above
    L2, a few hundred MB on the device: the size of the ncu captures); small: 32^2 x 256.
    Work units: pair-bins (aperture x surfel x bin) with the FP32 flop counts per
    pair-bin 16 (forward), 24 (JVP), 20 (VJP), 18 (correlation); the Gram as logical
    FP32 flops R S (S + 1).
    """
    import __graft_entry__

    __graft_entry__.build()
    from dsplat import FMCWConfig, FMCWModel, Scan
    from dsplat.certificate import fibonacci_sphere
    from dsplat.kernels import surfel as kernel
    from dsplat.kernels.gram import GramRows
    from dsplat.workloads import sphere_cap

    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    peaks, source = _peaks()
    small = args.case == "small"
    side, surfel_count = {"small": (32, 256), "medium": (64, 1000), "full": (128, 2000)}[args.case]
    config = FMCWConfig()
    positions, params, reflectivity = sphere_cap(side=side, surfel_count=surfel_count, device=device)
    centers, normals = params["centers"], params["normals"]
    A, S, K = len(positions), len(centers), config.num_range_bins
    generator = torch.Generator().manual_seed(0)
    weights = (reflectivity * params["areas"].sqrt()).to(torch.complex64)
    upstream = torch.complex(torch.randn(A, K, generator=generator), torch.randn(A, K, generator=generator)).to(device)
    dc = torch.randn(S, 3, generator=generator).to(device) * 1e-4
    dn = torch.randn(S, 3, generator=generator).to(device) * 1e-2
    dw = weights * 0.1
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    fp32_peak = 152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12  # nominal TFLOP/s
    rows = []

    def record(name, ms, units, flops_per_unit, unit="pair-bins"):
        achieved = units * flops_per_unit / (ms * 1e-3) / 1e12
        rows.append({"kernel": name, "ms": round(ms, 4), "units": units, "unit": unit,
                     "units_per_s": units / (ms * 1e-3), "achieved_tflops": round(achieved, 3),
                     "fp32_peak_tflops_nominal": round(fp32_peak, 1),
                     "frac_fp32": round(achieved / fp32_peak, 4)})  # fmt: skip

    it, wu = args.steps, args.warmup
    if args.only == "elimination":  # the pooled backward elimination alone (its ncu capture)
        _time_elimination(rows, S, generator, device, it, wu, flush)
        print(json.dumps({"case": args.case, "kernels": rows}), flush=True)
        return
    if args.only == "orient":  # the spatial search's normal-bank selection alone (its ncu capture)
        bank = fibonacci_sphere(24, device)
        ncand = 200000 if args.case == "full" else 50000
        grid = centers.repeat(ncand // S + 1, 1)[:ncand].contiguous()
        grid_n = normals.repeat(ncand // S + 1, 1)[:ncand].contiguous()
        grid_a = params["areas"].repeat(ncand // S + 1)[:ncand].contiguous()
        prop = positions[: min(A, 384)].contiguous()
        table = FMCWModel(Scan(upstream[: len(prop)], prop, config)).range_table(upstream[: len(prop)], 8)
        energy = upstream[: len(prop)].abs().square().sum().double()
        ms = _event_time(lambda: kernel.orient_best(config, prop, grid, grid_n, grid_a, bank, upstream[: len(prop)],
                                                    0.0, energy, True, table), it, wu, flush)  # fmt: skip
        record("dsg_surfel_orient_best", ms, len(prop) * len(grid) * 25, 12, "pair-normals")
        print(json.dumps({"case": args.case, "apertures": len(prop), "candidates": ncand, "kernels": rows}), flush=True)
        return
    ms = _event_time(lambda: kernel.render(config, positions, centers, normals, weights, 0.0), it, wu, flush)
    record("dsg_surfel_render", ms, A * S * K, 16)
    # the forward through the ADC samples: phasor recurrence (6 FP32 flops per pair-sample,
    # one anchor per lane and pair) plus the n_fft-point cuFFT, counted per pair-bin as above
    samples_only = _event_time(lambda: kernel.render_samples(config, positions, centers, normals, weights, 0.0),
                               it, wu, flush)  # fmt: skip
    record("dsg_surfel_render_samples (kernel alone)", samples_only, A * S * config.adc_samples, 6, "pair-samples")
    with kernel.render_form("samples"):
        ms = _event_time(lambda: kernel.render(config, positions, centers, normals, weights, 0.0), it, wu, flush)
    record("dsg_surfel_render [samples form + FFT]", ms, A * S * K, 16)
    ms = _event_time(lambda: kernel.jvp(config, positions, centers, normals, weights, dc, dn, dw, 0.0), it, wu, flush)
    record("dsg_surfel_jvp", ms, A * S * K, 24)
    ms = _event_time(lambda: kernel.vjp(config, positions, centers, normals, weights, upstream, 0.0), it, wu, flush)
    record("dsg_surfel_vjp", ms, A * S * K, 20)
    with kernel.correlation_form("exact"):
        ms = _event_time(lambda: kernel.vjp(config, positions, centers, normals, weights, upstream, 0.0), it, wu,
                         flush)  # fmt: skip
    record("dsg_surfel_vjp [exact bin sums]", ms, A * S * K, 20)
    if args.only == "splat":  # the three splat kernels alone (the ncu captures of render / JVP / VJP)
        print(json.dumps({"case": args.case, "apertures": A, "surfels": S, "bins": K, "kernels": rows}), flush=True)
        return
    sub = positions[: min(A, 768)].contiguous()
    cand = centers.repeat(max(1, 8192 // S), 1)[:8192].contiguous()
    cand_n = normals.repeat(max(1, 8192 // S), 1)[:8192].contiguous()
    for form, suffix in (("interp", ""), ("exact", " [exact bin sums]")):
        with kernel.correlation_form(form):
            ms = _event_time(lambda: kernel.correlate(config, sub, cand, cand_n, upstream[: len(sub)], 0.0), it, wu,
                             flush)  # fmt: skip
            record("dsg_surfel_correlate" + suffix, ms, len(sub) * len(cand) * K, 18)
            ms = _event_time(lambda: kernel.correlate_gradient(config, sub, cand[:1024], cand_n[:1024],
                                                               upstream[: len(sub)], 0.0, True), it, wu, flush)  # fmt: skip
            record("dsg_surfel_correlate_gradient" + suffix, ms, len(sub) * 1024 * K, 30)
    bank = fibonacci_sphere(24, device)
    ncand = 200000 if args.case == "full" else 50000
    grid = centers.repeat(ncand // S + 1, 1)[:ncand].contiguous()
    grid_n = normals.repeat(ncand // S + 1, 1)[:ncand].contiguous()
    prop = positions[: min(A, 384)].contiguous()
    table = FMCWModel(Scan(upstream[: len(prop)], prop, config)).range_table(upstream[: len(prop)], 8)
    ms = _event_time(lambda: kernel.correlate_orientations(config, prop, grid, grid_n, bank, upstream[: len(prop)],
                                                           0.0, table), it, wu, flush)  # fmt: skip
    record("dsg_surfel_correlate_orientations", ms, len(prop) * len(grid) * 25, 12, "pair-normals")
    # greedy separated peaks as a search level runs them: 1024 peaks kept from 1024 cubes of
    # 4^3 offsets (0.25 mm pitch) at separation 0.25 mm, scores in random order
    from dsplat.kernels import search

    cubes = centers.repeat(1024 // S + 1, 1)[:1024]
    axis = (torch.arange(4, device=device, dtype=torch.float32) - 1.5) * 2.5e-4
    offsets = torch.cartesian_prod(axis, axis, axis)
    points = (cubes[:, None, :] + offsets[None]).reshape(-1, 3).contiguous()
    scores = torch.rand(len(points), generator=torch.Generator().manual_seed(5)).to(device)
    ms = _event_time(lambda: search.peaks(scores, points, 1024, 2.5e-4), it, wu, flush)
    rows.append({"kernel": f"dsg_peaks ({len(points)} candidates, 1024 peaks, sort included)", "ms": round(ms, 4)})
    from dsplat.groundtruth import synthesize

    amplitudes = (reflectivity * params["areas"].sqrt()).to(torch.complex64)
    ms = _event_time(lambda: synthesize(positions, centers, normals, amplitudes, config), it, wu, flush)
    rows.append({"kernel": "synthesize (dsg_synthesize_adc float64 + range FFT)", "ms": round(ms, 3),
                 "units": A * S * config.adc_samples, "unit": "echo samples (float64)",
                 "units_per_s": A * S * config.adc_samples / (ms * 1e-3)})  # fmt: skip
    block = positions[: min(A, 125)].contiguous()
    ms = _event_time(lambda: kernel.design(config, block, centers, normals, params["areas"], 0.0, True), it, wu, flush)
    record("dsg_surfel_design", ms, len(block) * S * K, 10)
    from dsplat import DSFWConfig, ParameterConfig
    from dsplat.varpro import normal_equations
    from dsplat.workloads import box_of

    low, high = box_of(centers)
    model = FMCWModel(Scan(upstream, positions, config)).prepare({"centers": ParameterConfig(lower=low, upper=high)})
    # The fused design projection alone, on the first 2048 apertures with their block basis.
    from dsplat.kernels.gram import GramRows as _Rows
    from dsplat.kernels.gram import append_projected

    first = positions[: min(A, 2048)].contiguous()
    basis = model.block_basis(slice(0, len(first) * K))
    rank2 = basis.interleaved.shape[0]
    store = _Rows(S, len(first) * rank2, device)
    status = torch.zeros(1, dtype=torch.int32, device=device)

    def project_once():
        store.rows = 0
        append_projected(store, config, first, params, basis, 0.0, status)

    ms = _event_time(project_once, it, wu, flush)
    values = len(first) * S * K
    flops = values * 4 * rank2  # logical FP32 multiply-adds of U [rank2, 2K] . v, times 2
    tensor_peak = peaks["bf16_tflops"] / 3
    rows.append({"kernel": "dsg_design_project_bf16x3", "ms": round(ms, 4), "units": values,
                 "unit": "pair-bins (dictionary values)", "rank2": rank2, "units_per_s": values / (ms * 1e-3),
                 "achieved_tflops": round(flops / (ms * 1e-3) / 1e12, 2),
                 "tensor_peak_tflops": round(tensor_peak, 1),
                 "frac_tensor": round(flops / (ms * 1e-3) / 1e12 / tensor_peak, 4),
                 "out_gbs": round(2 * 2 * len(first) * rank2 * S / (ms * 1e-3) / 1e9, 1)})  # fmt: skip
    mixed = DSFWConfig(gram="bf16x3")
    ms = _event_time(lambda: normal_equations(model, params, upstream, mixed), it, wu, flush)
    rows.append({"kernel": "normal_equations (fused projection + tcgen05 Gram)", "ms": round(ms, 3)})
    ms = _event_time(lambda: normal_equations(model, params, upstream, DSFWConfig()), it, wu, flush)
    rows.append({"kernel": "normal_equations (FP32 design + projection + SSYRK)", "ms": round(ms, 3)})
    rows_r = {"small": 100_000, "medium": 200_000, "full": 400_000}[args.case]
    data = torch.randn(rows_r, S, generator=generator).to(device)
    store = GramRows(S, rows_r, device)
    store.append(data)
    total = torch.zeros((S, S), dtype=torch.float64, device=device)
    ms = _event_time(lambda: store.accumulate(total), it, wu, flush)
    logical = rows_r * S * (S + 1)
    achieved = logical / (ms * 1e-3) / 1e12
    tensor_peak = peaks["bf16_tflops"] / 3
    rows.append({"kernel": "dsg_gram_bf16x3", "ms": round(ms, 4), "units": logical, "unit": "logical FP32 flops",
                 "achieved_tflops": round(achieved, 2), "tensor_peak_tflops": round(tensor_peak, 1),
                 "frac_tensor": round(achieved / tensor_peak, 4),
                 "peak_source": f"{source} bf16_tflops (burst) / 3"})  # fmt: skip
    _time_elimination(rows, S, generator, device, it, wu, flush)
    # the spectral model on its 256^2 grid with 80 atoms: per-bin kernel (every atom at every
    # bin) against the separable form (per-axis tables and complex products)
    from dsplat import SpectralGrid
    from dsplat.kernels import spectral as spec

    sgrid = SpectralGrid((256, 256))
    sbins = sgrid.bins(device)
    scent = (torch.rand(80, 2, generator=generator) * 256).to(device)
    scoef = torch.complex(torch.randn(80, generator=generator), torch.randn(80, generator=generator)).to(device)
    sup = torch.complex(torch.randn(sgrid.size, generator=generator),
                        torch.randn(sgrid.size, generator=generator)).to(device)  # fmt: skip
    for label, fn in (("render, per-bin kernel", lambda: spec.render(sgrid, scent, scoef, sbins)),
                      ("render, separable", lambda: spec.render_grid(sgrid, scent, scoef)),
                      ("vjp, per-bin kernel", lambda: spec.vjp(sgrid, scent, scoef, sup, sbins)),
                      ("vjp, separable", lambda: spec.vjp_grid(sgrid, scent, scoef, sup))):  # fmt: skip
        ms = _event_time(fn, it, wu, flush)
        rows.append({"kernel": f"spectral {label} (256^2 bins, 80 atoms)", "ms": round(ms, 4)})
    print(json.dumps({"case": args.case, "apertures": A, "surfels": S, "bins": K, "kernels": rows}), flush=True)


def main():
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=5)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--mode", choices=["mixed", "plain"], default="mixed")
    parser.add_argument("--iterations", type=int, default=100, help="DSFW steps of the whole fit")
    parser.add_argument("--cpu-threads", type=int, default=None)
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparison run")
    parser.add_argument("--kernels", action="store_true", help="per-kernel roofline table instead")
    parser.add_argument("--case", choices=["small", "medium", "full"], default="full")
    parser.add_argument("--only", choices=["all", "splat", "orient", "elimination"], default="all",
                        help="with --kernels: which kernels")  # fmt: skip
    parser.add_argument("--accuracy", type=int, default=0, help="final-accuracy study of both arms on N seeds")
    parser.add_argument("--no-autotune", action="store_true", help="keep every launch shape automatic")
    parser.add_argument("--workload", choices=["sphere_cap", "uneven"], default="sphere_cap",
                        help="uneven: the 64-scene batch instead of the headline fit")
    parser.add_argument("--scenes", type=int, default=64)
    parser.add_argument("--rounds", type=int, default=10)
    args = parser.parse_args()
    if args.kernels:
        run_kernels(args)
        return
    if args.accuracy:
        run_accuracy(args)
        return
    if args.workload == "uneven":
        run_uneven(args)
        return
    world, rank, local = _distributed()
    if args.impl == "reference":
        result = run_reference(args, world, rank)
    else:
        result = run_ours(args, world, rank, local)
    if rank == 0 and result is not None:
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
