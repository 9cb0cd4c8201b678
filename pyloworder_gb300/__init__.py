"""GB300-native (sm_103a) implementation of pyLOM's SVD hot path.

A drop-in for ``pyLOM.math.tsqr_svd / randomized_svd / matmul`` and
``pyLOM.POD / DMD / SPOD.run``: same signatures, snapshot layout (points x
snapshots, one snapshot per column) and return tuples.  Python host code
drives hand-written CUDA kernels (libplom.so, C ABI in include/plom.h) on
PyTorch tensors; there is no CPU fallback.
"""
from . import vmmath
from . import vmmath as math
from . import POD
from . import DMD
from . import SPOD
from . import PCA

__version__ = "0.1.0"


def load_library():
    """Load (building in-tree if needed) libplom.so and return its handle."""
    from . import _lib
    return _lib.load()
