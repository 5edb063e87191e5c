"""GB300-native (sm_103a, FP64) eMix3d per-step hot path.

The compute lives in libemix_gb300.so (C ABI in include/emix_gb300.h);
``emix_gb300.ops`` mirrors the reference's operator interface over it,
``emix_gb300.fields`` generates the seeded synthetic workloads and
``emix_gb300.build`` compiles the library.
"""
from . import fields  # noqa: F401
