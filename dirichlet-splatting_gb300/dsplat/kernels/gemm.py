"""Row-basis projection products on the tensor cores with FP32-accurate BF16x9 emulation.

Inside `emulated()` (entered by the mixed-precision normal equations), RowBasis
products go through dsg_gemm_f32_bf16x9 (cuBLAS CUBLAS_COMPUTE_32F_EMULATED_16BFX9);
outside it they are plain FP32 matmuls, the reference's arithmetic.
"""

from __future__ import annotations

import threading
from contextlib import contextmanager

import torch

from . import _lib
from ._lib import call, ptr

_state = threading.local()


@contextmanager
def emulated(enabled=True):
    previous = getattr(_state, "on", False)
    _state.on = enabled
    try:
        yield
    finally:
        _state.on = previous


def project(matrix, rows):
    """matrix [m, k] @ rows [k, n] (FP32), emulated on the tensor cores when enabled."""
    if not getattr(_state, "on", False) or not rows.is_cuda or matrix.dtype != torch.float32:
        return matrix @ rows
    matrix, rows = matrix.contiguous(), rows.contiguous()
    m, k = matrix.shape
    n = rows.shape[1]
    out = torch.empty((m, n), dtype=torch.float32, device=rows.device)
    call("dsg_gemm_f32_bf16x9", m, n, k, ptr(matrix), k, ptr(rows), n, 0.0, ptr(out), n,
         _lib.stream(rows.device))  # fmt: skip
    return out
