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


def _inverse_scratch(n, element):
    """Largest k (n - k) product over the triangular inverse's halving (64-row leaves)."""
    if n <= 64:
        return 0
    k = (n // 2 + 63) // 64 * 64
    return max(k * (n - k) * element, _inverse_scratch(k, element), _inverse_scratch(n - k, element))


def test_triangular_inverse_workspace_covers_every_level():
    """The workspace holds the top level's product (the largest at every depth) and the
    zero-pivot word; no CUDA call is needed to size it."""
    from dsplat.kernels import _lib

    lib = _lib.library()
    assert lib.dsg_triangular_inverse_workspace_bytes(0, 0) == 0
    for n in list(range(1, 300)) + [511, 512, 513, 1000, 2256, 4097]:
        for complex_mode, element in ((0, 8), (1, 16)):
            need = (_inverse_scratch(n, element) + 255) // 256 * 256 + 4
            assert lib.dsg_triangular_inverse_workspace_bytes(n, complex_mode) >= need, (n, complex_mode)


def test_new_batched_entry_points_validate_on_the_host():
    """Bad widths, fraction counts and sizes return DSG_ERR_ARGUMENT (1) and a short
    workspace DSG_ERR_WORKSPACE (3) before anything touches the GPU."""
    from dsplat.kernels import _lib

    lib = _lib.library()
    fractions = (ctypes.c_float * 17)(*([1.0] * 17))
    fake = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    assert lib.dsg_trials(fake, fake, fake, fake, 4, 6, ctypes.addressof(fractions), 17, fake, fake, None) == 1
    assert lib.dsg_trials(fake, fake, fake, fake, 4, 5, ctypes.addressof(fractions), 8, fake, fake, None) == 1
    assert lib.dsg_ascent_partition(fake, fake, fake, fake, 1, fake, 4, fake, fake, 0, None, fake, fake, fake,
                                    fake, fake, None) == 1  # fmt: skip
    assert lib.dsg_ascent_partition(fake, fake, fake, fake, 1, fake, -1, fake, fake, 8, None, fake, fake, fake,
                                    fake, fake, None) == 1  # fmt: skip
    assert lib.dsg_ascent_select(fake, fake, fake, fake, 1, fake, 4, fake, fake, fake, fake, 17, None, fake, fake,
                                 1, fake, fake, fake, None) == 1  # fmt: skip
    spec = _lib.AscentSpec()
    spec.width = 4
    assert lib.dsg_ascent_update(ctypes.byref(spec), fake, fake, fake, fake, fake, fake, 1, 4, fake, fake, fake,
                                 fake, fake, fake, fake, fake, None) == 1  # fmt: skip
    spec.width, spec.scale[0] = 3, 0.0
    assert lib.dsg_ascent_update(ctypes.byref(spec), fake, fake, fake, fake, fake, fake, 1, 4, fake, fake, fake,
                                 fake, fake, fake, fake, fake, None) == 1  # fmt: skip
    info = ctypes.c_int32(0)
    assert lib.dsg_triangular_inverse(fake, -1, 0, None, 0, ctypes.byref(info), None) == 1
    assert lib.dsg_triangular_inverse(fake, 100, 0, None, 0, ctypes.byref(info), None) == 3
    assert lib.dsg_triangular_inverse(fake, 100, 0, fake, 8, ctypes.byref(info), None) == 3


def _prototypes():
    """{name: (return type, [parameter declarations])} of every entry point in the header."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"typedef struct\s*\{.*?\}\s*\w+\s*;", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)  # preprocessor lines (knob constants)
    found = {}
    for match in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(dsg_\w+)\s*\(([^)]*)\)\s*;", text):
        params = [p.strip() for p in match.group(3).split(",") if p.strip() and p.strip() != "void"]
        found[match.group(2)] = (" ".join(match.group(1).split()), params)
    return found


def test_bindings_match_the_header_prototypes():
    """Every ctypes signature has the header's parameter count, and pointer / integer /
    floating kinds agree position by position; return types map to int, size_t or char*."""
    from dsplat.kernels import _lib

    prototypes = _prototypes()
    assert set(prototypes) == set(declared())
    for name, (ret, params) in prototypes.items():
        restype, argtypes = _lib.SIGNATURES[name]
        assert len(argtypes) == len(params), (name, len(argtypes), params)
        for position, (declaration, kind) in enumerate(zip(params, argtypes, strict=True)):
            if "*" in declaration:
                assert kind is ctypes.c_void_p or issubclass(kind, ctypes._Pointer) or kind is ctypes.c_char_p, (
                    name, position, declaration, kind)  # fmt: skip
            elif declaration.startswith(("float", "const float")):
                assert kind is ctypes.c_float, (name, position, declaration)
            elif declaration.startswith(("double", "const double")):
                assert kind is ctypes.c_double, (name, position, declaration)
            elif declaration.startswith(("int64_t", "long long")):
                assert kind is ctypes.c_int64, (name, position, declaration)
            elif declaration.startswith("size_t"):
                assert kind is ctypes.c_size_t, (name, position, declaration)
            else:
                assert kind is ctypes.c_int32, (name, position, declaration)
        expected = {"int": ctypes.c_int, "size_t": ctypes.c_size_t, "const char*": ctypes.c_char_p,
                    "const char *": ctypes.c_char_p, "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64,
                    "int32_t": ctypes.c_int32,
                    "void": None}  # fmt: skip
        assert ret in expected, (name, ret)
        assert restype is expected[ret], (name, ret, restype)
