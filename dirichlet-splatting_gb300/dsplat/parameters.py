"""Per-atom parameter constraints: free components, step units and feasible sets.

Parameters are tensors with one row per atom (surfel centers [S, 3], normals [S, 3],
areas [S]). Solver steps are dimensionless; a ParameterConfig's scale converts them
to physical units, project restores feasibility and frozen components stay put.
Behaviour follows the reference's dsplat/parameters.py:15-83.
"""

from __future__ import annotations

from dataclasses import dataclass

import torch
import torch.nn.functional as F


_MASKS: dict = {}


@dataclass(frozen=True)
class ParameterConfig:
    trainable: bool | tuple[bool, ...] = True  # one flag, or one per component
    scale: float = 1.0  # physical length of one unit solver step
    lower: float | tuple[float, ...] | None = None
    upper: float | tuple[float, ...] | None = None
    period: tuple[float, ...] | None = None
    normalize: bool = False  # unit vectors (surfel normals)

    def mask(self, value):
        """Boolean mask of the free components of one row of value.

        Masks are cached per device and width, so that a loop captured in a CUDA graph
        never copies the flags from the host.
        """
        width = value.shape[1] if value.ndim == 2 else 1
        key = (self.trainable, value.device, width)
        flags = _MASKS.get(key)
        if flags is None:
            flags = torch.as_tensor(self.trainable, dtype=torch.bool, device=value.device).expand(width)
            _MASKS[key] = flags
        return flags

    def project(self, proposed, reference):
        """Closest feasible values to proposed; frozen components are taken from reference."""
        column = proposed.ndim == 1
        value = proposed[:, None] if column else proposed
        anchor = reference[:, None] if column else reference
        if self.period is not None:
            value = value.remainder(value.new_tensor(self.period))
        if self.lower is not None:
            value = torch.maximum(value, value.new_tensor(self.lower))
        if self.upper is not None:
            value = torch.minimum(value, value.new_tensor(self.upper))
        free = self.mask(reference)
        value = torch.where(free[None], value, anchor)
        if self.normalize and bool(free.any()):
            value = self._unit(value, anchor, free)
        return value[:, 0] if column else value

    @staticmethod
    def _unit(value, anchor, free):
        """Scale the free components so the row has unit length; frozen ones are kept."""
        fixed = torch.where(free[None], torch.zeros_like(value), value)
        moving = value - fixed
        # A free part of zero length borrows the reference's free direction.
        has_length = moving.norm(dim=-1, keepdim=True) > 0
        moving = torch.where(
            has_length, moving, torch.where(free[None], anchor, torch.zeros_like(anchor))
        )
        room = (1 - fixed.square().sum(-1, keepdim=True)).clamp(min=0).sqrt()
        length = moving.norm(dim=-1, keepdim=True)
        if bool(((room > 0) & (length == 0)).any()):
            raise ValueError("Cannot normalize a zero vector without a reference direction.")
        return fixed + moving * room / length.clamp(min=1e-30)

    def tangent(self, vector, value):
        """Part of an update [..., S, D] that project keeps at the unit vector value [S, D].

        Frozen components drop out, and so does the radial part of the free ones, whose
        squared length is one minus that of the frozen components.
        """
        if not self.normalize:
            return vector
        free = self.mask(value)
        moving = torch.where(free, value, torch.zeros_like(value))
        room = (1 - torch.where(free, torch.zeros_like(value), value).square().sum(-1, keepdim=True))
        room = room.clamp(min=0)
        vector = torch.where(free, vector, torch.zeros_like(vector))
        radial = (vector * moving).sum(-1, keepdim=True) * moving / room.clamp(min=1e-30)
        return torch.where(room > 0, vector - radial, torch.zeros_like(vector))

    def differential(self, jacobian, value):
        """Chain a dictionary derivative [..., S, D] through retraction, mask and scale."""
        if self.normalize:
            jacobian = self.tangent(jacobian, F.normalize(value, dim=-1))
        return jacobian[..., self.mask(value)] * self.scale


def periodic_delta(delta, period):
    """Differences folded into [-period/2, period/2] per axis; None leaves them unchanged."""
    if period is None:
        return delta
    period = torch.as_tensor(period, dtype=delta.dtype, device=delta.device)
    return delta - period * torch.round(delta / period)
