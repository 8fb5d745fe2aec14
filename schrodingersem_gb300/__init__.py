"""GB300-native (sm_103a) hot path of arotem3/SchrodingerSEM.

The CUDA library ``_lib/libsemgb300.so`` exports the C ABI declared in
``include/sem_gb300.h``; ``Context`` is a thin Python view of it used by
the tests and the benchmark.  There is no CPU fallback: every call runs in
the library's kernels, and a missing library raises.
"""
from .build import LIB, build  # noqa: F401
from . import meshgen  # noqa: F401


def Context(*args, **kwargs):  # noqa: N802 - mirrors the class name
    from .context import Context as _Context
    return _Context(*args, **kwargs)
