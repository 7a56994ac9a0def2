"""rc_gb300: GB300-native w-projection gridding / degridding.

A drop-in for the imaging hot path of SKA-ScienceDataProcessor/RC (MS5/MS6
DNA/Flow kernel bindings): the CUDA kernels and C ABI live in librc_gb300.so
(rc_gb300/csrc, include/rc_gb300.h); this package is its Python face.
"""
from . import lib  # noqa: F401

__all__ = ["lib", "build", "engine", "compat", "gcf", "synth"]
__version__ = "0.1.0"
