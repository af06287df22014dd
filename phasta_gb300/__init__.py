"""GB300-native drop-in for PHASTA's compressible matrix-free Newton-Krylov hot path.

The compute path is the CUDA library ``libphgpu.so`` (sources in ``csrc/``,
C ABI in ``include/phgpu.h``); ``solver.GpuSolver`` is the host-side mirror of
the reference routines (ElmMFG, ItrRes, i3LU, SolMFG, itrCorrect, the itrdrv
multi-corrector).  ``mesh`` generates the synthetic benchmark cases.
"""
from .mesh import Case, box, channel_case, periodic_vortex_case, uniform_state, vortex_state  # noqa: F401

__all__ = ["Case", "box", "channel_case", "periodic_vortex_case", "uniform_state", "vortex_state"]
