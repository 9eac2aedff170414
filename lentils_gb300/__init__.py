"""lentils_gb300: GB300 (sm_103a) implementation of Lentils' lensed visibility-space
operator chain -- Kaiser-Bessel NUFFT degridding/gridding, PEMD deflection and the
normal-equation operator of the CG source inversion -- behind the reference's C ABI
(include/lentils_gb300.h) and a Python mirror of its operator interface.

The CUDA library must be built (``lentils_gb300.build.build()``); importing the GPU entry
points without it raises, and nothing falls back to the CPU.
"""
from ._native import LentilsError, lib  # noqa: F401
from .spaces import FourierSpace, ImageSpace, Space, VisibilitySpace  # noqa: F401

__version__ = "0.1.0"
