"""GB300-native BLINK dirty-imaging path: phase corrections, nearest-neighbour uv gridding,
inverse 2D FFT, fftshift and normalisation, behind the C ABI in include/blink_imager_gb300.h.

The CUDA library is built in tree with ``python -m imager_gb300.build``; the Python layer
(:mod:`imager_gb300.imager`) calls it through ctypes and needs a CUDA device.
"""
__version__ = "0.1.0"
