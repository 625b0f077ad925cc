"""GB300-native structured-volume path of the Barney renderer.

Native library: barney_gb300/_lib/libbarney_gb300.so (C-ABI in include/).
"""
from . import _native  # noqa: F401

__all__ = ["_native"]
