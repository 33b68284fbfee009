"""GB300 (sm_103a) backend for ugsdr's acquisition-and-correlation path.

`ugsdr_gb300.api.Context` drives libugsdr_cuda.so (include/ugsdr_cuda.h);
`ugsdr_gb300.build` compiles it.  There is no CPU fallback.
"""
from . import _lib  # noqa: F401

__all__ = ["api", "build", "signals"]
