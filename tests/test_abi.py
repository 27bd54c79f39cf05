"""The C-ABI library builds, loads without a GPU and exports every declared entry point."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

HEADER = Path(__file__).resolve().parent.parent / "include" / "dsplat_gb300.h"


def declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dsg_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    from dsplat.kernels import _lib

    lib = _lib.library()
    names = declared()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_version_and_error_strings_need_no_gpu():
    from dsplat.kernels import _lib

    lib = _lib.library()
    assert b"sm_103a" in lib.dsg_version()
    assert lib.dsg_error_string(3) == b"workspace missing or too small"


def test_invalid_arguments_are_rejected_before_any_launch():
    """Validation happens on the host: bad sizes return codes, nothing is launched."""
    from dsplat import FMCWConfig
    from dsplat.kernels import _lib

    lib = _lib.library()
    chirp = _lib.chirp(FMCWConfig())
    assert lib.dsg_surfel_render(ctypes.byref(chirp), None, -1, None, None, None, 1, None, None, 0,
                                 None) == 1  # fmt: skip
    odd = _lib.chirp(FMCWConfig(pad_factor=3))
    assert lib.dsg_surfel_render(ctypes.byref(odd), None, 1, None, None, None, 1, None, None, 0,
                                 None) == 2  # fmt: skip
    assert lib.dsg_surfel_render_workspace_bytes(ctypes.byref(chirp), 1024, 256) > 0
    assert lib.dsg_surfel_render_workspace_bytes(ctypes.byref(chirp), 16384, 2000) == 0
    assert lib.dsg_surfel_correlate_gradient(ctypes.byref(chirp), None, 1, None, None, 1, None, 4,
                                             None, None, None, None, None, 0, None) == 1  # fmt: skip
    assert lib.dsg_peaks(None, None, None, 1, 9, 1, 0.0, None, None) == 1
    assert lib.dsg_peaks(None, None, None, 1, 3, 5000, 0.0, None, None) == 1


def test_cpu_tensors_are_refused():
    import pytest
    import torch

    from dsplat import FMCWConfig
    from dsplat.kernels import DsplatKernelError
    from dsplat.kernels import surfel as kernel

    with pytest.raises(DsplatKernelError, match="CUDA"):
        kernel.render(FMCWConfig(), torch.zeros(4, 3), torch.zeros(2, 3), torch.zeros(2, 3),
                      torch.ones(2, dtype=torch.complex64), 0.0)  # fmt: skip
