"""GB300-native (sm_103a) implementation of raypier's non-sequential ray-tracing
hot path.

The modules mirror the reference's ``raypier.core`` names so that a caller of
``raypier.core.ctracer.trace_segment`` / ``raypier.core.tracer.trace_rays`` can
switch imports:

    from raypier_optics_gb300 import ctracer, cfaces, cmaterials, cshapes, cdistortions
    from raypier_optics_gb300.tracer import trace_rays

All tracing runs in ``librp_gb300.so`` (C ABI: include/rp_gb300.h); there is no
CPU fallback.
"""
from . import _native  # noqa: F401
from . import ctracer, cshapes, cfaces, cmaterials, cdistortions, tracer  # noqa: F401

__all__ = ["ctracer", "cshapes", "cfaces", "cmaterials", "cdistortions", "tracer"]
