"""GB300-native DEM time-step engine with the behaviour of the reference DEM code (IAries/VEDO).

The product is the CUDA engine in ``csrc/`` behind the C ABI of ``include/vedo_gpu.h``
(built into ``vedo_gb300/_build/libvedogpu.so``); this package holds the scene model, the
reference ``.ido`` format, seeded synthetic scenes and a thin ctypes binding.
"""
from .scene import Scene  # noqa: F401

__version__ = "0.1.0"
