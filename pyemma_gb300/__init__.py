"""GB300-native k-means discretization with PyEMMA's call signatures.

``pyemma_gb300.coordinates`` mirrors ``pyemma.coordinates.cluster_kmeans``
and ``assign_to_centers``; the arithmetic runs in hand-written sm_103a CUDA
kernels behind the C ABI of ``libkmgpu.so`` (include/kmgpu.h).
"""
__version__ = "0.1.0"

from . import coordinates  # noqa: E402,F401
from .serialization import list_models, load  # noqa: E402,F401
