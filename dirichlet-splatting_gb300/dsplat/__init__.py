"""Dirichlet splatting on GB300: the render-and-fit path as sm_103a CUDA kernels.

A drop-in for the reference package `dsplat` on its render-and-fit path:

parameters  per-atom parameter constraints
spectral    Dirichlet atoms on a spectral grid
surfel      oriented surfels: scattering and the area chain around the kernels
fmcw        FMCW sensor, scans and the surfel measurement model
groundtruth planar arrays and FMCW scans synthesized from the beat signal
dsfw        the solver loop over varpro, certificate, replacement, refinement, spatial
kernels     the CUDA kernels (libdsplat_gb300.so, C ABI include/dsplat_gb300.h)
"""

from .certificate import CertificateSearchConfig
from .dsfw import DSFWConfig, fit, initialize, step
from .fmcw import FMCWConfig, FMCWModel, Scan
from .parameters import ParameterConfig
from .spatial import SpatialSearchConfig
from .spectral import SpectralGrid, SpectralModel

__all__ = [
    "CertificateSearchConfig",
    "DSFWConfig",
    "FMCWConfig",
    "FMCWModel",
    "ParameterConfig",
    "Scan",
    "SpatialSearchConfig",
    "SpectralGrid",
    "SpectralModel",
    "fit",
    "initialize",
    "step",
]
__version__ = "0.1.0"
