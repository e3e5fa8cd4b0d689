"""rskel: GB300-native recursive-skeletonization solver (Python side).

The solver itself is the CUDA/C++ library ``lib/librskel.so`` behind the C
ABI in ``include/rskel.h``; this package holds its ctypes binding
(:mod:`rskel.capi`), the seeded boundary generators (:mod:`rskel.geometry`)
and the build step (:mod:`rskel.build`).
"""
from . import geometry  # noqa: F401
