"""Streamed normal equations G = A^H A / M, q = A^H y / M of one support.

The dictionary A (M observations x S atoms; 33.5 GB at 16 384 apertures x 2000 surfels)
is never stored: rows are generated in blocks of whole apertures, projected onto the
row basis of their range band, reduced into the Gram, and dropped. Two accumulators:

  Fp32Syrk       the reference's arithmetic (dsplat/varpro.py:91-120): each real block
                 adds its upper triangle in float32 (SSYRK), folded into a float64 total
                 every FOLD blocks; complex blocks use complex GEMMs.
  TensorCoreGram split-BF16x3 on tcgen05 (DSFWConfig.gram == "bf16x3", real
                 coefficients): every projected row block is stored transposed as bf16
                 hi + lo, in the fused design-projection kernel when the basis allows
                 (no dictionary block ever reaches HBM), and one tcgen05 launch adds the
                 whole Gram to the float64 total.

The right-hand side of the fused path is the correlation of every atom with the data
(dsg_surfel_correlate), which needs no dictionary rows either.
"""

from __future__ import annotations

import torch

from .kernels.cublas import syrk

FOLD = 8  # float32 blocks summed before each float64 fold of the Gram


def row_chunk(model, columns, config):
    """Observation rows per streamed block: at most dictionary_elements / columns, whole apertures."""
    limit = min(config.row_chunk, max(1, config.dictionary_elements // columns))
    align = model.row_alignment
    return max(align, limit - limit % align)


def _block_ranges(model, chunk):
    for start in range(0, model.size, chunk):
        yield slice(start, min(start + chunk, model.size))


def projected_rows(model, chunk):
    """Real rows that model.blocks(..., real=True, chunk) yields, known before streaming."""
    if not hasattr(model, "block_basis"):
        return 2 * model.size
    bins = model.shape[1]
    total = 0
    for rows in _block_ranges(model, chunk):
        basis = model.block_basis(rows)
        width = 2 * bins if basis is None else basis.interleaved.shape[0]
        total += width * (-(-rows.stop // bins) - rows.start // bins)
    return total


def fused_rows(model, params, store, chunk, first_unknown=0):
    """Store every projected real row block with the fused design-projection kernel.

    Consecutive blocks sharing one basis go to the kernel as one aperture range. Returns
    the kernel status tensor, or None (nothing stored) when the model or a block's basis
    is outside what the kernel covers; the caller then streams explicit blocks. With
    first_unknown > 0 params' surfels fill the store's rows from there, beside unknowns
    stored before with the same model and chunk (the same reduction rows).
    """
    from .kernels.gram import append_projected, fused_supported

    if not hasattr(model, "block_basis"):
        return None
    config, positions = model.sensor
    bins = model.shape[1]
    runs = []  # [first aperture, stop aperture, basis]
    for rows in _block_ranges(model, chunk):
        basis = model.block_basis(rows)
        if not fused_supported(config, basis):
            return None
        first, stop = rows.start // bins, rows.stop // bins
        if runs and runs[-1][2] is basis and runs[-1][1] == first:
            runs[-1][1] = stop
        else:
            runs.append([first, stop, basis])
    status = torch.zeros(1, dtype=torch.int32, device=positions.device)
    row = 0
    for first, stop, basis in runs:
        row = append_projected(store, config, positions[first:stop], params, basis, model.fresnel_n, status,
                               first_unknown=first_unknown, row=row)  # fmt: skip
    if first_unknown == 0:
        store.rows = row
    elif row != store.rows:
        raise RuntimeError("projected rows do not line up with the stored unknowns")
    return status


class ProjectionCache:
    """Projected rows (bf16 hi/lo) of the latest supports, reused when a pool extends one.

    The merged replacement pools the support with new candidates. When the support's rows
    were stored by an earlier normal-equation pass of the same model over the very same
    parameter tensors (states never write their tensors in place, so identity means equal
    values), only the candidates are projected, into the rows after the support's, with
    that pass's block layout. After a replacement the survivors' rows are moved into their
    slots (adopt) so the next step's pool finds the new support. Only models registered
    with track (the fitted states' models, not their aperture subsets) are kept; holds the
    last LIMIT stores (a few GB each at 16 384 apertures).
    """

    LIMIT = 3
    MODELS = 4

    def __init__(self):
        self.entries = []  # [model, params (the tensors), store, chunk], most recent last
        self.models = []

    def track(self, model):
        """Keep the projected rows of this model's normal equations from now on."""
        if not any(m is model for m in self.models):
            self.models.append(model)
            del self.models[: -self.MODELS]
            self.entries = [e for e in self.entries if any(m is e[0] for m in self.models)]

    def tracks(self, model):
        return any(m is model for m in self.models)

    def put(self, model, params, store, chunk):
        if not self.tracks(model):
            return None
        self.entries = [e for e in self.entries if e[2] is not store]
        self.entries.append([model, dict(params), store, chunk])
        del self.entries[: -self.LIMIT]
        return self.entries[-1]

    def find(self, model, params):
        """The entry of model whose stored rows are those of params, or None.

        The same tensors match at once; otherwise equal values do (one device read), as
        when a caller copies the previous state's parameters in again; the entry then
        takes the caller's tensors.
        """
        mine = [e for e in reversed(self.entries) if e[0] is model and e[1].keys() == params.keys()]
        for entry in mine:
            if all(entry[1][key] is params[key] for key in params):
                return entry
        for entry in mine:
            shaped = all(entry[1][key].shape == params[key].shape and entry[1][key].dtype == params[key].dtype
                         and entry[1][key].device == params[key].device for key in params)  # fmt: skip
            if shaped:
                equal = torch.stack([(entry[1][key] == params[key]).all() for key in params]).all()
                if bool(equal):
                    entry[1] = dict(params)
                    return entry
        return None

    def adopt(self, entry, slots, owners, params):
        """The stored support after a replacement: slot j takes the pooled row slots[j]."""
        store = entry[2]
        if len(owners):
            sources = slots[owners]
            store.hi.index_copy_(0, owners, store.hi.index_select(0, sources))
            store.lo.index_copy_(0, owners, store.lo.index_select(0, sources))
        store.set_columns(len(slots))
        entry[1] = dict(params)
        self.entries = [e for e in self.entries if e is not entry] + [entry]  # by identity: models hold tensors

    def clear(self):
        self.entries = []
        self.models = []


PROJECTIONS = ProjectionCache()


def _symmetrize_upper(total, size):
    """Full symmetric matrix from the upper triangle of total, divided by size."""
    upper = torch.triu(total)
    return (upper + torch.triu(total, 1).mT) / size


class Fp32Syrk:
    """Float32 SSYRK per block, folded into float64 every FOLD blocks."""

    def __init__(self, count, device):
        self.total = torch.zeros((count, count), dtype=torch.float64, device=device)
        self.part = torch.zeros((count, count), dtype=torch.float32, device=device)
        self.rhs = torch.zeros(count, dtype=torch.float64, device=device)
        self.blocks = 0

    def add(self, a, y):
        a = a.contiguous()
        syrk(a, self.part)
        self.rhs += a.T @ y
        self.blocks += 1
        if self.blocks % FOLD == 0:
            self.total += self.part
            self.part.zero_()

    def finish(self):
        self.total += self.part
        return self.total, self.rhs


class TensorCoreGram:
    """Split-BF16x3 rows stored for one tcgen05 Gram launch (real coefficients).

    store, when given, is a GramRows already holding rows (ProjectionCache); reserve
    allocates room for that many more unknowns.
    """

    def __init__(self, model, count, chunk, device, store=None, reserve=0):
        from .kernels.gram import GramRows

        if store is None:
            store = GramRows(count, projected_rows(model, chunk), device, reserve=reserve)
        else:
            store.set_columns(count)
        self.store = store
        self.total = torch.zeros((count, count), dtype=torch.float64, device=device)
        self.rhs = torch.zeros(count, dtype=torch.float64, device=device)

    def add(self, a, y):
        self.store.append(a)
        self.rhs += a.T @ y

    def finish(self, column_from=0, deferred=False):
        """(total, rhs); deferred also returns the Gram's status word unread (else checked)."""
        from .kernels.gram import check

        status = self.store.accumulate(self.total, column_from=column_from)
        if deferred:
            return self.total, self.rhs, status
        check(status)
        return self.total, self.rhs


def normal_equations(model, params, target, config, deferred=False):
    """(G, q) = (A^H A / M, A^H y / M) of params, streamed over projected row blocks.

    Real coefficients return float32 real G and q (float64 accumulation inside);
    complex coefficients return complex G and q accumulated in complex64. deferred returns
    ((G, q), statuses) without reading anything back: the kernels' status words, which
    the caller checks (kernels.gram.check) before it uses G and q.
    """
    statuses = []
    out = _normal_equations(model, params, target, config, statuses)
    if deferred:
        return out, statuses
    from .kernels.gram import check

    for status in statuses:
        check(status)
    return out


def _normal_equations(model, params, target, config, statuses):
    count = len(params["centers"])
    chunk = row_chunk(model, count, config)
    if not config.real:
        gram = target.new_zeros((count, count))
        rhs = target.new_zeros(count)
        for a, y in model.blocks(params, target, False, chunk):
            gram.addmm_(a.mH, a)
            rhs.addmv_(a.mH, y)
        return (gram + gram.mH) / (2 * model.size), rhs / model.size
    device = target.device
    if getattr(config, "gram", "fp32") == "bf16x3":
        merged = getattr(config, "replacement", "merged") == "merged" and PROJECTIONS.tracks(model)
        acc = TensorCoreGram(model, count, chunk, device, reserve=config.batch if merged else 0)
        status = fused_rows(model, params, acc.store, chunk)
        if status is None:
            for a, y in model.blocks(params, target, True, chunk):
                acc.add(a, y)
        else:
            acc.rhs += model.correlate(params, target)[0].real.double()
            statuses.append(status)
            if merged:
                PROJECTIONS.put(model, params, acc.store, chunk)
        total, rhs, gram_status = acc.finish(deferred=True)
        statuses.append(gram_status)
    else:
        acc = Fp32Syrk(count, device)
        for a, y in model.blocks(params, target, True, chunk):
            acc.add(a, y)
        total, rhs = acc.finish()
    return _symmetrize_upper(total, model.size).float(), (rhs / model.size).float()
