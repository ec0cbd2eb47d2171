"""GB300 (sm_103a) implementation of EdelweissFE's NIST/NISTParallel hot path.

The element loop, the VIJ->CSR scatter and the Krylov solve run as hand-written
CUDA kernels in ``libefgpu.so`` (C ABI: ``include/efgpu.h``); this package holds
the ctypes binding and the host-side mirror of the reference's Newton driver.
"""

from .exceptions import CutbackRequest, DivergingSolution, ReachedMaxIterations, StepFailed  # noqa: F401

__all__ = ["CutbackRequest", "DivergingSolution", "ReachedMaxIterations", "StepFailed"]
