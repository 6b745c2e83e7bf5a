"""GB300 (sm_103a) isosurface extraction: Flying Edges and Marching Cubes.

A drop-in for miniIsosurface's serial extraction calls.  The compute lives
in libminiiso.so (hand-written CUDA kernels behind a C ABI, include/miniiso.h);
this package is the host-side mirror of the reference interface.
"""
from .api import (FLYING_EDGES, MARCHING_CUBES, MC_DUPFREE, Batch, Context, DeviceMesh, FlyingEdgesAlgorithm,
                  Image3D, MarchingCubes, Request, TriangleMesh, bad_format, batch_lanes, count_device,
                  default_context, extract, extract_batch, extract_typed, extract_device, file_not_found,
                  generate_blobs, generate_value_noise, loadImage, make_grid, saveImage, saveTriangleMesh,
                  set_batch_graph, set_batch_lanes, set_batch_split, batch_split, set_graph, set_batch_fused,
                  PackedBuffers, PackedMesh, extract_batch_packed, batch_fused_split)
from .builder import build, library_path

__all__ = [
    "FLYING_EDGES", "MARCHING_CUBES", "MC_DUPFREE", "Batch", "Context", "DeviceMesh", "FlyingEdgesAlgorithm",
    "Image3D", "MarchingCubes", "Request", "TriangleMesh", "bad_format", "batch_lanes", "build", "count_device",
    "default_context", "extract", "extract_batch", "extract_typed", "set_batch_graph", "set_batch_lanes",
    "set_batch_split", "batch_split", "set_graph", "set_batch_fused", "PackedBuffers",
    "extract_batch_packed", "batch_fused_split", "PackedMesh",
    "extract_device", "file_not_found", "generate_blobs", "generate_value_noise", "library_path", "loadImage",
    "make_grid", "saveImage", "saveTriangleMesh",
]
