"""mepgl_gb300 -- GB300-native hot path of the gauged string method (mepgl).

The compute path is the CUDA library ``libmepgl_gb300.so`` (hand-written
sm_103a kernels behind a C ABI, include/mepgl.h).  It is loaded lazily by
:func:`mepgl_gb300.native.lib`, which raises when the library is missing:
there is no CPU fallback.
"""
from .problem import Problem, StringState, neighbour_codes  # noqa: F401

__all__ = ["Problem", "StringState", "neighbour_codes"]
