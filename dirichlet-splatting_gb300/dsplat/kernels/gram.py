"""Split-BF16x3 Gram products on the tcgen05 tensor cores (the mixed-precision path).

GramRows collects projected real design rows [m, S] block by block, each stored
transposed and split into bf16 hi + lo (dsg_split_transpose_bf16); accumulate() then
adds PT PT^T to a float64 [S, S] total in one tcgen05 launch (dsg_gram_bf16x3, plus an
ordered sum of its K-split parts), so the whole streamed normal-equation Gram is one dense
contraction, bitwise reproducible. The plain path is
cublas.syrk (FP32 SSYRK), as in the reference's dsplat/varpro.py:108-118.
"""

from __future__ import annotations

import torch

from . import _lib
from ._lib import DsplatKernelError, call, ptr

SM_COUNT = 152


def _round_up(value, step):
    return -(-value // step) * step


def tile_pairs(n_pad, column_from=0):
    """Number of upper-triangle 128 x 128 tiles whose column tile is at least column_from's."""
    tiles, first = n_pad // 128, column_from // 128
    band = tiles - first
    return first * band + band * (band + 1) // 2


def k_splits(n_pad, k_pad, column_from=0):
    """CTAs per output tile: fill the GPU in whole waves, each share at least 16 stages."""
    pairs = tile_pairs(n_pad, column_from)
    stages = k_pad // 64
    best = 1
    for splits in range(1, max(1, stages // 16) + 1):
        ctas = pairs * splits
        if ctas >= 4 * SM_COUNT:
            break
        best = splits
    # round the CTA count up to a whole wave when that keeps every share >= 16 stages
    ctas = pairs * best
    waves = -(-ctas // SM_COUNT)
    exact = waves * SM_COUNT
    if exact % pairs == 0 and stages // (exact // pairs) >= 16:
        best = exact // pairs
    return max(1, best)


class GramRows:
    """Transposed bf16 hi/lo storage of up to `capacity` real rows of `columns` unknowns.

    reserve adds storage for that many more unknowns (set_columns widens to them later
    without moving the stored ones; the Gram only ever covers the current columns).
    """

    def __init__(self, columns, capacity, device, reserve=0):
        self.k_pad = _round_up(max(capacity, 1), 64)
        self.n_alloc = _round_up(max(columns + reserve, 1), 128)
        self.hi = torch.empty((self.n_alloc, self.k_pad), dtype=torch.bfloat16, device=device)
        self.lo = torch.empty_like(self.hi)
        self.set_columns(columns)
        self.rows = 0

    def set_columns(self, columns):
        """Cover `columns` unknowns (at most the allocated ones); stored rows stay."""
        if _round_up(max(columns, 1), 128) > self.n_alloc:
            raise DsplatKernelError("GramRows column capacity exceeded")
        self.columns = columns
        self.n_pad = _round_up(max(columns, 1), 128)

    def append(self, block):
        """Store block [m, columns] (FP32) as the next m reduction indices."""
        block = block.to(torch.float32).contiguous()
        m = block.shape[0]
        if self.rows + m > self.k_pad:
            raise DsplatKernelError("GramRows capacity exceeded")
        call(
            "dsg_split_transpose_bf16", ptr(block), m, self.columns, self.rows, ptr(self.hi),
            ptr(self.lo), self.k_pad, _lib.stream(block.device),
        )  # fmt: skip
        self.rows += m

    def accumulate(self, total, column_from=0, splits=None):
        """total [S, S] float64 += upper tiles of the stored rows' Gram (unused tail is zeroed).

        column_from > 0 computes only the tiles that hold columns >= column_from. splits
        overrides the K-split count (default: the autotuner's value for this shape, else
        k_splits).
        """
        if self.rows < self.k_pad:
            self.hi[: self.n_pad, self.rows :].zero_()
            self.lo[: self.n_pad, self.rows :].zero_()
        if self.n_pad > self.columns:
            self.hi[self.columns : self.n_pad].zero_()
            self.lo[self.columns : self.n_pad].zero_()
        k_pad = _round_up(max(self.rows, 1), 64)
        status = torch.zeros(1, dtype=torch.int32, device=total.device)
        hi, lo = self.hi[: self.n_pad, :k_pad], self.lo[: self.n_pad, :k_pad]
        if k_pad != self.k_pad:  # a narrower view needs contiguous rows for the tensor map
            hi, lo = hi.contiguous(), lo.contiguous()
        # logical FP32 flops of the needed symmetric block (a SYRK count)
        added = self.columns - int(column_from)
        _lib.add_work("dsg_gram_bf16x3", float(self.rows) * added * (2 * int(column_from) + added + 1))
        if splits is None:
            from .. import autotune

            automatic = k_splits(self.n_pad, k_pad, column_from)
            splits = autotune.gram_splits(automatic, autotune.gram_key(self.n_pad, k_pad, column_from, total.device))
        nbytes = _lib.query("dsg_gram_bf16x3_workspace_bytes", self.n_pad, k_pad, int(column_from), int(splits))
        work, nbytes = _lib.workspace(nbytes, total.device)
        call(
            "dsg_gram_bf16x3", ptr(hi), ptr(lo), self.columns, self.n_pad, k_pad, int(column_from),
            int(splits), ptr(total), total.shape[1], ptr(work), nbytes, ptr(status), _lib.stream(total.device),
        )  # fmt: skip
        return status


_SPLIT_BASES: dict = {}


def split_basis(interleaved):
    """bf16 hi/lo [128, 2K] of an interleaved row basis [2 rank, 2K] (rows past 2 rank zero)."""
    key = (interleaved.data_ptr(), tuple(interleaved.shape), interleaved.device)
    entry = _SPLIT_BASES.get(key)
    if entry is None:
        rank2, width = interleaved.shape
        padded = torch.zeros((128, width), dtype=torch.float32, device=interleaved.device)
        padded[:rank2] = interleaved
        hi = padded.to(torch.bfloat16)
        lo = (padded - hi.float()).to(torch.bfloat16)
        entry = (hi.contiguous(), lo.contiguous(), interleaved)  # keep the source alive
        _SPLIT_BASES[key] = entry
    return entry[0], entry[1]


def fused_supported(config, basis):
    """Whether dsg_design_project_bf16x3 covers this chirp and basis."""
    return (basis is not None and basis.interleaved.shape[0] <= 128
            and config.num_range_bins in (32, 64, 128) and config.pad_factor in (1, 2, 4))  # fmt: skip


def append_projected(store, config, positions, params, basis, fresnel_n, status, first_unknown=0, row=None):
    """Store the basis-projected real dictionary rows of apertures `positions` (fused kernel).

    The unknowns (params' surfels) fill the store's rows from first_unknown; the reduction
    index starts at row (default: after the stored rows, which then advance).
    """
    from . import _lib as lib

    hi, lo = split_basis(basis.interleaved)
    rank2 = basis.interleaved.shape[0]
    count = len(positions) * rank2
    start = store.rows if row is None else row
    if start + count > store.k_pad or first_unknown + len(params["centers"]) > store.n_alloc:
        raise DsplatKernelError("GramRows capacity exceeded")
    positions = positions.to(torch.float32).contiguous()
    centers = params["centers"].to(torch.float32).contiguous()
    normals = params["normals"].to(torch.float32).contiguous()
    areas = params["areas"].to(torch.float32).contiguous()
    from .. import autotune

    autotune.apply("project", surfels=len(params["centers"]), bins=config.num_range_bins, pad=config.pad_factor,
                   rank2=rank2, device=positions.device)  # fmt: skip
    # logical FP32 flops of the projection U [rank2, 2K] . v over every aperture-surfel pair
    lib.add_work("dsg_design_project_bf16x3",
                 float(len(positions)) * len(centers) * 2 * (2 * config.num_range_bins) * rank2)  # fmt: skip
    call(
        "dsg_design_project_bf16x3", lib.chirp(config, fresnel_n), ptr(positions), len(positions),
        ptr(centers), ptr(normals), ptr(areas), len(centers), ptr(hi), ptr(lo), rank2,
        ptr(store.hi[first_unknown:]), ptr(store.lo[first_unknown:]), store.k_pad, start, ptr(status),
        lib.stream(positions.device),
    )  # fmt: skip
    if row is None:
        store.rows += count
    return start + count


def check(status):
    """Raise if the Gram kernel reported a bounded wait that ran out (reads one int)."""
    if int(status.item()) != 0:
        raise DsplatKernelError("dsg_gram_bf16x3: a bounded wait ran out")


def gram_accumulate(rows, total):
    """total [S, S] float64 += upper tiles of rows^T rows for one block rows [m, S]."""
    store = GramRows(rows.shape[1], rows.shape[0], rows.device)
    store.append(rows)
    check(store.accumulate(total))
