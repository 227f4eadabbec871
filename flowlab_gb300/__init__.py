"""flowlab_gb300 — a GB300-native (sm_103a) engine for flowlab's 2D
incompressible MAC-grid projection step.

The compute lives in hand-written CUDA behind a C ABI
(include/flowlab_gb300.h, built into flowlab_gb300/_lib/libflowlab_gb300.so).
This package holds the host side: the ctypes binding (`native`), the mirror of
the reference's GpuStep / PressureSolver / Advector seams (`engine`) and the
scene builders (`scenes`). Importing it does not load the CUDA library; the
first engine object does, and raises if the library is missing.
"""
__all__ = ["scenes", "native", "engine"]
