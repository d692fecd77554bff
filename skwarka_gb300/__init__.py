"""GB300-native ray-query and light-transport path of the Skwarka renderer.

The compute path is the in-tree CUDA library ``_lib/libskw.so`` (C ABI in
``include/skw.h``); this package is its host-side mirror of the reference
interfaces.  Importing it does not load the library; the first query does,
and fails loudly if it was not built.
"""
from .accel import Context, Primitive, TriangleAccelerator, TriangleMesh, default_context, unpack_hits
from .kdtree import PhotonKDTree, compress_direction, direction_table

__all__ = ["Context", "Primitive", "TriangleAccelerator", "TriangleMesh", "default_context", "unpack_hits",
           "PhotonKDTree", "compress_direction", "direction_table"]
