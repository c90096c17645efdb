"""GB300-native spatial statistics for atom-probe ion clouds.

The CUDA kernels and the C ABI live in paraprobe_gb300/csrc (declared in
include/paraprobe_gb300.h); `paraprobe_gb300.native` binds them with ctypes.
"""
from . import native, synth  # noqa: F401

__all__ = ["native", "synth"]
