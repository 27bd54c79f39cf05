"""Per-atom parameter constraints: which components move, in what unit, inside which set.

An atom field is a tensor with one row per atom (surfel centers [S, 3], normals [S, 3],
areas [S]; a 1-D field is handled as one column). The solver works in dimensionless
steps; a ParameterConfig turns them into physical units (scale), keeps the result
feasible (project: periodic wrap, box, unit length) and leaves frozen components alone.
Semantics of the reference's dsplat/parameters.py:15-83; every constraint tensor is
built once per (device, width) so that nothing is copied from the host inside a
captured CUDA graph.
"""

from __future__ import annotations

from dataclasses import dataclass

import torch

# (what, value, device, width, dtype) -> device tensor of a constraint
_CONSTANTS: dict = {}


def _constant(what, value, like, width):
    """A cached [width] tensor of value (a flag, a number or a per-component tuple)."""
    frozen_value = tuple(value) if isinstance(value, list) else value
    key = (what, frozen_value, like.device, width, like.dtype if what != "free" else torch.bool)
    found = _CONSTANTS.get(key)
    if found is None:
        dtype = torch.bool if what == "free" else like.dtype
        found = torch.as_tensor(value, dtype=dtype, device=like.device).expand(width).clone()
        _CONSTANTS[key] = found
    return found


def _rows(x):
    """x as a 2-D [atoms, components] view and a function restoring the original rank."""
    if x.ndim == 1:
        return x[:, None], lambda y: y[:, 0]
    return x, lambda y: y


@dataclass(frozen=True)
class ParameterConfig:
    trainable: bool | tuple[bool, ...] = True  # one flag, or one per component
    scale: float = 1.0  # physical length of one unit solver step
    lower: float | tuple[float, ...] | None = None
    upper: float | tuple[float, ...] | None = None
    period: tuple[float, ...] | None = None
    normalize: bool = False  # unit vectors (surfel normals)

    @property
    def any_free(self):
        """Whether any component is trainable, decided on the host."""
        flags = self.trainable
        return any(flags) if isinstance(flags, (tuple, list)) else bool(flags)

    def mask(self, value):
        """Boolean [components] mask of the free components of a row of value."""
        return _constant("free", self.trainable, value, value.shape[1] if value.ndim == 2 else 1)

    def free_index(self, value):
        """Long [free components] indices of the free components (gathers without a device read)."""
        width = value.shape[1] if value.ndim == 2 else 1
        flags = self.trainable if isinstance(self.trainable, (tuple, list)) else (self.trainable,) * width
        key = ("index", tuple(bool(f) for f in flags), value.device, width)
        found = _CONSTANTS.get(key)
        if found is None:
            found = torch.tensor([i for i in range(width) if flags[i]], dtype=torch.long, device=value.device)
            _CONSTANTS[key] = found
        return found

    def project(self, proposed, reference):
        """The feasible point nearest proposed; frozen components come from reference."""
        x, restore = _rows(proposed)
        anchor, _ = _rows(reference)
        width = x.shape[1]
        if self.period is not None:
            x = torch.remainder(x, _constant("period", self.period, x, width))
        if self.lower is not None or self.upper is not None:
            low = None if self.lower is None else _constant("lower", self.lower, x, width)
            high = None if self.upper is None else _constant("upper", self.upper, x, width)
            x = torch.clamp(x, min=low, max=high)
        free = self.mask(reference)
        x = torch.where(free, x, anchor)
        if self.normalize and self.any_free:
            x = _onto_sphere(x, anchor, free)
        return restore(x)

    def tangent(self, vector, value):
        """The part of an update [..., S, D] that survives projection at unit vectors value.

        Frozen components are dropped; on the unit sphere, so is the component along the
        free part of value (its free part has squared length one minus the frozen part's).
        """
        if not self.normalize:
            return vector
        free = self.mask(value)
        along = torch.where(free, value, 0.0)
        slack = (1 - (value - along).square().sum(-1, keepdim=True)).clamp(min=0)
        moved = torch.where(free, vector, 0.0)
        radial = along * ((moved * along).sum(-1, keepdim=True) / slack.clamp(min=1e-30))
        return torch.where(slack > 0, moved - radial, 0.0)

    def differential(self, jacobian, value):
        """Chain a derivative [..., S, D] through the sphere retraction, the mask and the scale."""
        if self.normalize:
            unit = value / value.norm(dim=-1, keepdim=True).clamp(min=1e-12)
            jacobian = self.tangent(jacobian, unit)
        return jacobian[..., self.mask(value)] * self.scale


def _onto_sphere(x, anchor, free):
    """Rescale the free components of each row so the row has unit length.

    The frozen components keep their values and leave 1 - |frozen|^2 of squared length to
    the free ones; a row whose free part is zero takes the anchor's free direction.
    """
    frozen = torch.where(free, 0.0, x)
    moving = x - frozen
    empty = moving.norm(dim=-1, keepdim=True) == 0
    moving = torch.where(empty, torch.where(free, anchor, 0.0), moving)
    room = (1 - frozen.square().sum(-1, keepdim=True)).clamp(min=0).sqrt()
    length = moving.norm(dim=-1, keepdim=True)
    if bool(((room > 0) & (length == 0)).any()):
        raise ValueError("Cannot normalize a zero vector without a reference direction.")
    return frozen + moving * (room / length.clamp(min=1e-30))


def periodic_delta(delta, period):
    """Differences folded into [-period/2, period/2] per axis; None leaves them as they are."""
    if period is None:
        return delta
    p = torch.as_tensor(period, dtype=delta.dtype, device=delta.device)
    return delta - p * torch.round(delta / p)
