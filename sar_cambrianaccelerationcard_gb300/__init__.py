"""GB300-native SAR back-projection imager (host side).

The compute path is the C-ABI library ``libsarbp.so`` (CUDA for sm_103a) built
from ``csrc/``; this package holds its ctypes binding, the synthetic scene
definitions and the image-quality metrics.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes"]
