"""aurora_gb300: GB300-native (sm_103a) rendering hot path of the Aurora renderer.

The product is the CUDA shared library aurora_gb300/_build/libaurora_gb300.so
with the C ABI of include/aurora_gb300.h. This package holds its build recipe
(build.py), a ctypes front end (api.py), the ABI struct dtypes (types.py) and
the seeded workload generators (scenes.py).
"""
from . import types  # noqa: F401

__all__ = ["types"]
