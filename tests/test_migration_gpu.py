"""The range-migration initializer (dsplat.fmcw.migration) against the reference's own.

tests/golden/reference_migration.npz holds a 16 x 16 raster scan synthesized by the
reference's groundtruth.synthesize and the focusing strengths its migration
(dsplat/fmcw.py:361-454) returns at a plane of points and at four regular depth planes;
the GPU version (the focusing sum in dsg_migration_focus) must reproduce them.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch
from conftest import rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_migration.npz")


@pytest.mark.parametrize("name", ["plane", "volume"])
def test_migration_matches_the_reference(name):
    """float32 arithmetic in a different summation order: rel-L2 within 1e-4."""
    from dsplat import FMCWConfig, Scan
    from dsplat.fmcw import migration

    scan = Scan(torch.from_numpy(GOLDEN["data"]).cuda(), torch.from_numpy(GOLDEN["positions"]).cuda(), FMCWConfig())
    points = torch.from_numpy(GOLDEN[f"{name}_points"]).cuda()
    strength = migration(scan, points, (16, 16), padding=int(GOLDEN[f"{name}_padding"][0]))
    expected = torch.from_numpy(GOLDEN[f"{name}_strength"])
    assert strength.shape == expected.shape
    assert rel_l2(strength, expected) < 1e-4

