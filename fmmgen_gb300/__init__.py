"""GB300 (sm_103a) octree FMM evaluation pass behind rpep/fmmgen's operator
surface: the device octree + interaction lists of the example tree code, the
P2M/M2M/M2L/L2L/L2P/P2P sweeps, and the generated operators as batched device
calls.  Compute runs in libfmmgen_gb300.so (hand-written CUDA); this package is
the host-side binding.
"""
from ._lib import FMMError, lib  # noqa: F401
from .tree import Tree, build_forest, build_tree, direct  # noqa: F401
from . import operators  # noqa: F401
from .demag import DemagFMM  # noqa: F401
from .pipeline import stream_compute  # noqa: F401

__all__ = ["Tree", "build_forest", "build_tree", "direct", "operators", "DemagFMM", "FMMError", "lib",
           "stream_compute"]
