"""GB300-native FFT-VIE operator and GMRES solver for MARIE's pure-VIE path.

The compute path is libmarie_gb300.so (hand-written sm_103a CUDA behind a C
ABI, include/marie_gb300.h); this package is the Python host side: the ctypes
binding, an operator class, a mirror of the reference's function-handle
interface and seeded synthetic inputs.
"""
from ._build import build  # noqa: F401
from . import _lib  # noqa: F401
from .operator import VieOperator, assemble_green, SolveReport  # noqa: F401
from . import phantoms  # noqa: F401

__all__ = ["build", "VieOperator", "assemble_green", "SolveReport", "phantoms"]
