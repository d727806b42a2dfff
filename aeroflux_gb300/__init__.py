"""aeroflux_gb300: GB300 (sm_103a) engine for AeroFlux's fractional-step hot path.

The compute path is libaeroflux_cuda (C ABI, include/aeroflux_cuda.h); this
package mirrors the reference's Go API on top of it.
"""
from ._lib import (AF_ADVECTION_MACCORMACK, AF_ADVECTION_SEMI_LAGRANGIAN, AF_PRECISION_FP64,  # noqa: F401
                   AF_PRECISION_MIXED)
from .engine import (AerofluxError, Config, Engine, FaultError, Field, Mesh,  # noqa: F401
                     MACBytes, New)
