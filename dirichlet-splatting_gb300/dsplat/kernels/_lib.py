"""ctypes binding of libdsplat_gb300.so, the C ABI declared in include/dsplat_gb300.h.

The library is built from dsplat/csrc on first use (see dsplat/build.py). Every call
passes raw device pointers of CUDA tensors and torch's current stream; a nonzero
return code raises DsplatKernelError. There is no CPU path: a tensor that is not on
a CUDA device raises before anything launches.
"""

from __future__ import annotations

import ctypes
import threading
from functools import cache

import torch

from .. import build as _build


class DsplatKernelError(RuntimeError):
    """A kernel entry point returned an error code, or the library is unavailable."""


class Chirp(ctypes.Structure):
    _fields_ = [
        ("num_bins", ctypes.c_int32),
        ("n_fft", ctypes.c_int32),
        ("samples", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("k0_per_meter", ctypes.c_double),
        ("fc", ctypes.c_double),
        ("slope", ctypes.c_double),
        ("t_start", ctypes.c_double),
        ("lambda_m", ctypes.c_double),
        ("c0", ctypes.c_double),
        ("fresnel_n", ctypes.c_double),
    ]


class RenderScene(ctypes.Structure):
    _fields_ = [
        ("chirp", Chirp),
        ("positions", ctypes.c_void_p),
        ("apertures", ctypes.c_int32),
        ("centers", ctypes.c_void_p),
        ("normals", ctypes.c_void_p),
        ("weights", ctypes.c_void_p),
        ("surfels", ctypes.c_int32),
        ("out", ctypes.c_void_p),
    ]


class Grid(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("nfft", ctypes.c_int32 * 3),
        ("samples", ctypes.c_int32 * 3),
        ("window", ctypes.c_int32),
        ("max_taps", ctypes.c_int32),
        ("radius", ctypes.c_float),
    ]


P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
F32 = ctypes.c_float
F64 = ctypes.c_double
SZ = ctypes.c_size_t
class AscentSpec(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32),
        ("normalize", ctypes.c_int32 * 2),
        ("scale", ctypes.c_float * 2),
        ("mask", ctypes.c_float * 6),
    ]


CP = ctypes.POINTER(Chirp)
RSP = ctypes.POINTER(RenderScene)
AP = ctypes.POINTER(AscentSpec)
GP = ctypes.POINTER(Grid)

# name: (restype, argtypes); the order and types follow include/dsplat_gb300.h.
SIGNATURES = {
    "dsg_version": (ctypes.c_char_p, []),
    "dsg_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "dsg_launch_count": (ctypes.c_uint64, []),
    "dsg_tuning_set": (ctypes.c_int, [I32, I32]),
    "dsg_tuning_get": (I32, [I32]),
    "dsg_surfel_render_workspace_bytes": (SZ, [CP, I32, I32]),
    "dsg_surfel_render": (ctypes.c_int, [CP, P, I32, P, P, P, I32, P, P, SZ, P]),
    "dsg_surfel_render_samples_workspace_bytes": (SZ, [CP, I32, I32]),
    "dsg_surfel_render_samples": (ctypes.c_int, [CP, P, I32, P, P, P, I32, P, P, SZ, P, P]),
    "dsg_surfel_render_scenes_workspace_bytes": (SZ, [RSP, I32]),
    "dsg_surfel_render_scenes": (ctypes.c_int, [RSP, I32, P, SZ, P, P]),
    "dsg_surfel_jvp": (ctypes.c_int, [CP, P, I32, P, P, P, P, P, P, I32, P, P, SZ, P]),
    "dsg_surfel_reduce_workspace_bytes": (SZ, [CP, I32, I32, I32]),
    "dsg_surfel_vjp": (ctypes.c_int, [CP, P, I32, P, P, P, I32, P, P, P, P, P, SZ, P]),
    "dsg_surfel_vjp_fixed_scratch": (ctypes.c_int, [CP, P, I32, P, P, P, I32, P, P, P, P, P]),
    "dsg_surfel_interp_tables": (ctypes.c_int, [I32, I32, P, SZ, P, SZ]),
    "dsg_surfel_residual_tables_bytes": (SZ, [CP, I32, I32]),
    "dsg_surfel_residual_tables": (ctypes.c_int, [CP, P, I32, I32, P, SZ, P]),
    "dsg_surfel_tabled_workspace_bytes": (SZ, [I32, I32, I32]),
    "dsg_surfel_correlate_tabled": (ctypes.c_int, [CP, P, I32, P, P, I32, P, P, I32, P, P, P, SZ, P]),
    "dsg_surfel_correlate_gradient_tabled": (ctypes.c_int, [CP, P, I32, P, P, I32, P, I32, P, P, P, P, P, SZ, P]),
    "dsg_surfel_correlate": (ctypes.c_int, [CP, P, I32, P, P, I32, P, P, P, P, SZ, P]),
    "dsg_surfel_correlate_active": (ctypes.c_int, [CP, P, I32, P, P, I32, P, P, I32, P, P, P, SZ, P]),
    "dsg_surfel_correlate_gradient": (
        ctypes.c_int,
        [CP, P, I32, P, P, I32, P, I32, P, P, P, P, P, SZ, P],
    ),
    "dsg_surfel_correlate_orientations": (
        ctypes.c_int,
        [CP, P, I32, P, P, I32, P, I32, P, P, P, I32, P, P],
    ),
    "dsg_surfel_orient_best": (ctypes.c_int, [CP, P, I32, P, P, P, I32, P, I32, P, P, P, I32, P, I32, P, P, P]),
    "dsg_surfel_design": (ctypes.c_int, [CP, P, I32, P, P, P, I32, I32, P, P]),
    "dsg_surfel_jacobian": (ctypes.c_int, [CP, P, I32, P, P, I32, P, P, P]),
    "dsg_spectral_axis_tables": (ctypes.c_int, [GP, P, P, I32, P, P, P]),
    "dsg_spectral_render": (ctypes.c_int, [GP, P, P, I32, P, P, I32, P, P]),
    "dsg_spectral_jvp": (ctypes.c_int, [GP, P, P, I32, P, P, P, P, I32, P, P]),
    "dsg_spectral_vjp_workspace_bytes": (SZ, [GP, I32, I32]),
    "dsg_spectral_vjp": (ctypes.c_int, [GP, P, P, I32, P, P, P, I32, P, P, P, SZ, P]),
    "dsg_spectral_design": (ctypes.c_int, [GP, P, P, I32, P, I32, P, P, P]),
    "dsg_range_gate": (ctypes.c_int, [P, I32, P, I32, P, I32, F32, I32, P, P]),
    "dsg_peaks": (ctypes.c_int, [P, P, P, I32, I32, I32, F32, P, P]),
    "dsg_distinct": (ctypes.c_int, [P, P, P, I32, I32, P, I32, P, F32, I32, P, P, P]),
    "dsg_elimination_workspace_bytes": (SZ, [I32, I32, I32]),
    "dsg_synthesize_adc": (ctypes.c_int, [CP, F64, P, I32, P, P, P, I32, P, P]),
    "dsg_migration_focus": (ctypes.c_int, [P, I32, I32, I32, P, P, P, I32, I32, P, I32, P, P]),
    "dsg_backward_elimination": (ctypes.c_int, [P, P, I32, I32, P, I64, I32, P, SZ, P, P]),
    "dsg_backward_elimination_factor": (ctypes.c_int, [P, P, I32, I32, P, I64, I32, P, SZ, P, P]),
    "dsg_triangular_inverse_workspace_bytes": (SZ, [I32, I32]),
    "dsg_triangular_inverse": (ctypes.c_int, [P, I32, I32, P, SZ, P, P]),
    "dsg_direction": (ctypes.c_int, [P, P, P, P, I32, I32, F32, P, P]),
    "dsg_trial": (ctypes.c_int, [P, P, P, P, I32, I32, F32, P, P, P]),
    "dsg_trials": (ctypes.c_int, [P, P, P, P, I32, I32, P, I32, P, P, P]),
    "dsg_ascent_partition": (ctypes.c_int, [P, P, P, P, I32, P, I32, P, P, I32, P, P, P, P, P, P, P]),
    "dsg_ascent_select": (ctypes.c_int, [P, P, P, P, I32, P, I32, P, P, P, P, I32, P, P, P, I32, P, P, P, P]),
    "dsg_ascent_update": (ctypes.c_int, [AP, P, P, P, P, P, P, I32, I32, P, P, P, P, P, P, P, P, P]),
    "dsg_energy_workspace_bytes": (SZ, [I64]),
    "dsg_energy": (ctypes.c_int, [P, P, I64, P, P, SZ, P]),
    "dsg_range_response": (ctypes.c_int, [F64, F64, I32, I32, I32, I32, P, P]),
    "dsg_syrk_f32": (ctypes.c_int, [P, I64, I32, P, P]),
    "dsg_gemm_f32_bf16x9": (ctypes.c_int, [I32, I32, I32, P, I32, P, I32, F32, P, I32, P]),
    "dsg_design_project_bf16x3": (
        ctypes.c_int,
        [CP, P, I32, P, P, P, I32, P, P, I32, P, P, I64, I64, P, P],
    ),
    "dsg_split_transpose_bf16": (ctypes.c_int, [P, I64, I32, I64, P, P, I64, P]),
    "dsg_gram_bf16x3_workspace_bytes": (SZ, [I32, I64, I32, I32]),
    "dsg_gram_bf16x3": (ctypes.c_int, [P, P, I32, I32, I64, I32, I32, P, I32, P, SZ, P, P]),
}

_lock = threading.Lock()


@cache
def library() -> ctypes.CDLL:
    """The loaded library; builds it first when a source is newer than the binary."""
    with _lock:
        try:
            path = _build.build()
        except Exception as error:  # the CUDA path has no substitute
            raise DsplatKernelError(f"cannot build libdsplat_gb300.so: {error}") from error
        try:
            lib = ctypes.CDLL(str(path))
        except OSError as error:
            raise DsplatKernelError(f"cannot load {path}: {error}") from error
        for name, (restype, argtypes) in SIGNATURES.items():
            function = getattr(lib, name)
            function.restype = restype
            function.argtypes = argtypes
        return lib


# Optional per-entry-point timing: name -> list of (start, end) CUDA events. Set to a
# dict to record; None (the default) records nothing.
TIMERS: dict | None = None
# Kernel launches replayed from CUDA graphs (the library's own counter sees a captured
# launch once, at capture time).
REPLAYED_LAUNCHES = 0
# Optional algorithmic work per entry point (flops or bytes, as each caller defines),
# accumulated while TIMERS is recording.
WORK: dict = {}


def add_work(name: str, units: float) -> None:
    if TIMERS is not None:
        WORK[name] = WORK.get(name, 0.0) + float(units)


def call(name: str, *args) -> None:
    """Invoke one entry point and raise on a nonzero status."""
    if TIMERS is not None:
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        status = getattr(library(), name)(*args)
        end.record()
        TIMERS.setdefault(name, []).append((start, end))
    else:
        status = getattr(library(), name)(*args)
    if status != 0:
        message = library().dsg_error_string(status).decode()
        raise DsplatKernelError(f"{name} failed with status {status}: {message}")


def query(name: str, *args) -> int:
    return int(getattr(library(), name)(*args))


def ptr(tensor: torch.Tensor | None):
    """Device pointer of a contiguous CUDA tensor (None for a missing optional buffer)."""
    if tensor is None:
        return None
    if not tensor.is_cuda:
        raise DsplatKernelError("dsplat kernels take CUDA tensors; there is no CPU path")
    if not tensor.is_contiguous():
        raise DsplatKernelError("dsplat kernels take contiguous tensors")
    return ctypes.c_void_p(tensor.data_ptr())


def stream(device: torch.device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def workspace(nbytes: int, device: torch.device) -> tuple[torch.Tensor | None, int]:
    """A scratch buffer from torch's caching allocator (safe inside graph capture)."""
    if nbytes <= 0:
        return None, 0
    return torch.empty(nbytes, dtype=torch.uint8, device=device), nbytes


def chirp(config, fresnel_n: float = 0.0) -> Chirp:
    """C struct of an FMCWConfig (dsplat.fmcw.FMCWConfig) and the surfel material."""
    return Chirp(
        num_bins=config.num_range_bins,
        n_fft=config.n_fft,
        samples=config.adc_samples,
        pad=config.pad_factor,
        k0_per_meter=1.0 / config.range_bin_spacing_m,
        fc=config.fc_hz,
        slope=config.slope_hz_s,
        t_start=config.adc_start_time_s,
        lambda_m=config.lambda_m,
        c0=config.c0_m_s,
        fresnel_n=float(fresnel_n),
    )


def real_view(value: torch.Tensor) -> torch.Tensor:
    """Interleaved (re, im) float32 view [..., 2] of a complex tensor, contiguous."""
    value = value.to(torch.complex64).resolve_conj().resolve_neg()
    return torch.view_as_real(value.contiguous()).contiguous()


def f32(value: torch.Tensor) -> torch.Tensor:
    return value.to(torch.float32).contiguous()
