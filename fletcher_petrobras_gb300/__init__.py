"""GB300 (sm_103a) Fletcher TTI pseudo-acoustic propagator.

The product is libfletcher_gb300.so (include/fletcher_gb300.h): the
reference's DRIVER_* back-end interface over hand-written CUDA kernels.  This
package builds it in-tree and binds it with ctypes.
"""
from .build import build, LIB as LIB_PATH  # noqa: F401
from .driver import FletcherError, Propagator  # noqa: F401
from .models import C0, C1, C2, Problem  # noqa: F401
