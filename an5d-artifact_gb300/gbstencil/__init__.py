"""gbstencil: GB300-native temporally-blocked stencil engine for the AN5D
artifact's stencil time loops (star2d/3d r1-4, box2d/3d r1-4, j2d5pt, j2d9pt,
j2d9pt-gol, j3d27pt, gradient2d; float and double).

The engine itself is ``_lib/libgbstencil.so`` (C ABI in include/gbstencil.h);
this package is its Python host side: the ctypes binding (``capi``), the
device-grid helpers (``grid``) and the build driver (``build``).
"""
from . import capi  # noqa: F401
from .capi import GbsError, kernel_stencil, NAMES  # noqa: F401
