"""ctypes binding of include/miniiso.h (libminiiso.so, built in-tree).

The library is the product: if it is missing this module raises instead of
falling back to anything else.
"""
import ctypes as C
from pathlib import Path

from . import builder as _build

ISO_OK = 0
ISO_ERR_INVALID_ARG = 1
ISO_ERR_OOM = 2
ISO_ERR_CUDA = 3
ISO_ERR_CAPACITY = 4
ISO_ERR_OVERFLOW = 5
ISO_ERR_TIMEOUT = 6
ISO_ERR_IO = 7
ISO_ERR_FORMAT = 8
ISO_ERR_STATE = 9
ISO_ERR_TOO_LARGE = 10
ISO_NOALLOC_MAX_ROWS = 1 << 20
ISO_NOALLOC_MAX_ROW_POINTS = 858993459

PASS_NAMES = ("classify", "count", "scan", "fe_generate", "mc_vertices", "mc_triangles", "vertices")

ISO_FLYING_EDGES = 0
ISO_MARCHING_CUBES = 1
ISO_MC_DUPFREE = 2

# iso_dtype
ISO_FLOAT32, ISO_INT8, ISO_UINT8, ISO_INT16, ISO_UINT16, ISO_INT32, ISO_FLOAT64 = range(7)


class IsoGrid(C.Structure):
    _fields_ = [("dims", C.c_int64 * 3), ("spacing", C.c_float * 3), ("origin", C.c_float * 3)]


class IsoMesh(C.Structure):
    _fields_ = [("points", C.c_void_p), ("normals", C.c_void_p), ("tris", C.c_void_p),
                ("index_bytes", C.c_int32), ("cap_points", C.c_int64), ("cap_tris", C.c_int64),
                ("n_points", C.c_int64), ("n_tris", C.c_int64)]


class IsoBlockSet(C.Structure):
    _fields_ = [("stats", C.c_void_p), ("n_blocks", C.c_int64), ("isoval", C.c_float)]


class IsoRequest(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("grid", IsoGrid), ("isoval", C.c_float), ("algorithm", C.c_int32)]


# name -> (restype, argtypes); mirrors include/miniiso.h
SIGNATURES = {
    "iso_status_string": (C.c_char_p, [C.c_int]),
    "iso_version": (C.c_char_p, []),
    "iso_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "iso_ctx_destroy": (C.c_int, [C.c_void_p]),
    "iso_ctx_last_error": (C.c_char_p, [C.c_void_p]),
    "iso_ctx_scratch_bytes": (C.c_int64, [C.c_void_p]),
    "iso_ctx_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_ctx_profile_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "iso_count_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_float,
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]),
    "iso_count_device_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_float, C.c_void_p,
                                           C.c_void_p]),
    "iso_count_slab": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_int64, C.c_int64,
                                 C.c_float, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]),
    "iso_extract_slab": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_int64, C.c_int64,
                                   C.c_float, C.c_int64, C.c_int64, C.POINTER(IsoMesh), C.c_void_p]),
    "iso_extract_device_typed": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(IsoGrid), C.c_float,
                                           C.POINTER(IsoMesh), C.c_void_p]),
    "iso_extract_host_typed": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(IsoGrid), C.c_float,
                                         C.POINTER(IsoMesh), C.c_void_p]),
    "iso_extract_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_float,
                                     C.POINTER(IsoMesh), C.c_void_p]),
    "iso_extract_device_async": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_float,
                                           C.POINTER(IsoMesh), C.c_void_p, C.c_void_p]),
    "iso_extract_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(IsoGrid), C.c_float,
                                   C.POINTER(IsoMesh), C.c_void_p]),
    "iso_extract_batch": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(IsoRequest), C.POINTER(IsoMesh),
                                    C.POINTER(C.c_int), C.c_void_p]),
    "iso_extract_batch_packed": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(IsoRequest), C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int), C.c_void_p]),
    "iso_count_batch": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(IsoRequest), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64), C.POINTER(C.c_int), C.c_void_p]),
    "iso_batch_set_lanes": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_batch_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_batch_set_fused": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_batch_fused_split": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "iso_ctx_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_ctx_set_narrow": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_batch_set_split": (C.c_int, [C.c_void_p, C.c_int]),
    "iso_batch_split": (C.c_int, [C.c_void_p]),
    "iso_block_count": (C.c_int64, [C.POINTER(IsoGrid)]),
    "iso_block_stats": (C.c_int, [C.c_void_p, C.POINTER(IsoGrid), C.c_void_p, C.c_void_p]),
    "iso_block_tris": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(IsoGrid), C.c_float, C.c_void_p, C.c_void_p]),
    "iso_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "iso_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_void_p]),
    "iso_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_void_p]),
    "iso_mlp_predict": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(IsoBlockSet), C.c_void_p, C.c_void_p]),
    "iso_batch_lanes": (C.c_int, [C.c_void_p]),
    "iso_fe_create": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(IsoGrid), C.c_float, C.POINTER(C.c_void_p)]),
    "iso_fe_pass1": (C.c_int, [C.c_void_p]),
    "iso_fe_pass2": (C.c_int, [C.c_void_p]),
    "iso_fe_pass3": (C.c_int, [C.c_void_p]),
    "iso_fe_pass4": (C.c_int, [C.c_void_p]),
    "iso_fe_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "iso_fe_grid_edges": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "iso_fe_move_output": (C.c_int, [C.c_void_p, C.POINTER(IsoMesh)]),
    "iso_fe_destroy": (C.c_int, [C.c_void_p]),
    "iso_vtk_read_image": (C.c_int, [C.c_char_p, C.POINTER(IsoGrid), C.c_void_p]),
    "iso_vtk_write_mesh": (C.c_int, [C.c_char_p, C.POINTER(IsoMesh)]),
    "iso_vtk_write_image": (C.c_int, [C.c_char_p, C.POINTER(IsoGrid), C.c_void_p]),
    "iso_generate_blobs": (C.c_int, [C.POINTER(C.c_int64), C.c_int, C.c_uint64, C.c_void_p]),
    "iso_generate_value_noise": (C.c_int, [C.POINTER(C.c_int64), C.c_int, C.c_int, C.c_uint64, C.c_void_p]),
}

_LIB = None


def library_path():
    return _build.library_path()


def load():
    """Load libminiiso.so.  Raises RuntimeError when it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = Path(library_path())
    if not path.exists():
        raise RuntimeError("libminiiso.so is not built (%s); run miniisosurface_gb300.builder.build() "
                           "or __graft_entry__.build()" % path)
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class IsoError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = load().iso_status_string(status).decode()
        super().__init__("%s%s" % (msg, (": " + what) if what else ""))


def check(status, ctx=None):
    if status != ISO_OK:
        what = ""
        if ctx:
            what = (load().iso_ctx_last_error(ctx) or b"").decode()
        raise IsoError(status, what)
