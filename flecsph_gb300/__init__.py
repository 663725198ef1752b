"""GB300-native SPH particle hot path (FleCSPH body-system / physics surface).

The compute path is libfsph_gb300.so (hand-written CUDA for sm_103a behind
the C ABI in include/fsph.h); ``BodySystem`` is its Python host mirror.
"""
from . import abi  # noqa: F401
from .abi import FsphError, Params  # noqa: F401


def BodySystem(*args, **kw):  # noqa: N802 - mirrors the reference class name
    from .sph import BodySystem as _BS
    return _BS(*args, **kw)
