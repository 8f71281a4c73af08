"""GB300-native residual engine for ibis's compressible finite-volume path.

The residual (MUSCL reconstruction with Barth-Jespersen limiting, Hanel /
AUSMDV / LDFSS2 / Rusanov fluxes, least-squares gradients, viscous fluxes,
face-to-cell accumulation) and the explicit Runge-Kutta update built on it run
as hand-written sm_103a CUDA kernels behind the C ABI of libibisgb.so
(include/ibisgb.h).  This package holds the host-side mirror of ibis's
interface (``Simulation``), the grid/config generators of the benchmark cases
(``grids``) and the build recipe (``build``).
"""
from .simulation import Batch, Simulation  # noqa: F401

__all__ = ["Batch", "Simulation"]
