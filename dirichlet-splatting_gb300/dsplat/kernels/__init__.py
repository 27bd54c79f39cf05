"""CUDA kernels of the render-and-fit path and their PyTorch bindings.

Each module mirrors one binding module of the reference's dsplat/kernels package:
surfel (FMCW profiles, derivatives, dictionary rows and correlations), spectral,
search, reduce, response and cublas. All of them call libdsplat_gb300.so, the sm_103a
library whose C ABI is include/dsplat_gb300.h; _lib holds the ctypes binding.
Tensors are CUDA float32, complex values complex64, and complex gradients follow the
PyTorch convention dL/dx = Re(conj(upstream) * dy/dx).
"""

from ._lib import DsplatKernelError, library

__all__ = ["DsplatKernelError", "library"]
