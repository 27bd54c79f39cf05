"""Symmetric rank-k update of the streamed normal equations (replaces the reference's
dsplat/kernels/cublas.py ctypes call; here cuBLAS is linked into libdsplat_gb300.so)."""

from __future__ import annotations

from . import _lib
from ._lib import call, ptr


def syrk(rows, out):
    """Add rows^T rows to the upper triangle of out [n, n]; the lower triangle is untouched."""
    rows = rows.contiguous()
    count, columns = rows.shape
    call("dsg_syrk_f32", ptr(rows), count, columns, ptr(out), _lib.stream(rows.device))
