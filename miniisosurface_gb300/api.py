"""Host-side mirror of miniIsosurface's extraction interface over the C ABI.

Reference names are kept so that code written against the reference reads the
same:

  util::Image3D            -> Image3D          (flyingEdges/util/Image3D.h:26-85)
  util::TriangleMesh       -> TriangleMesh     (flyingEdges/util/TriangleMesh.h:24-90)
  FlyingEdgesAlgorithm     -> FlyingEdgesAlgorithm, pass1()..pass4(), moveOutput()
                              (flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49)
  MarchingCubes(image, v)  -> MarchingCubes     (marchingCubes/serial/main.cpp:42-44)
  util::loadImage          -> loadImage         (flyingEdges/util/LoadImage.h:168-198)
  util::saveTriangleMesh   -> saveTriangleMesh  (flyingEdges/util/SaveTriangleMesh.h:33-118)

All compute runs in libminiiso.so on the GPU; there is no CPU path.  IO
errors raise file_not_found / bad_format like util/Errors.h:26-48.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import IsoGrid, IsoMesh, check, load

FLYING_EDGES = _lib.ISO_FLYING_EDGES
MARCHING_CUBES = _lib.ISO_MARCHING_CUBES
MC_DUPFREE = _lib.ISO_MC_DUPFREE  # MC, vertices in global-edge-index order (marchingCubes/openmpDupFree)


class file_not_found(FileNotFoundError):
    """util::file_not_found (flyingEdges/util/Errors.h:26-36)."""


class bad_format(ValueError):
    """util::bad_format (flyingEdges/util/Errors.h:38-48)."""


def _algo(a):
    if a in (FLYING_EDGES, "fe", "flying_edges", "FlyingEdges"):
        return FLYING_EDGES
    if a in (MARCHING_CUBES, "mc", "marching_cubes", "MarchingCubes"):
        return MARCHING_CUBES
    if a in (MC_DUPFREE, "mc_dupfree", "dupfree"):
        return MC_DUPFREE
    raise ValueError("unknown algorithm %r" % (a,))


def _ptr(x):
    """Address of a numpy array or torch tensor (host or device)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


_DTYPES = {"float32": _lib.ISO_FLOAT32, "int8": _lib.ISO_INT8, "uint8": _lib.ISO_UINT8, "int16": _lib.ISO_INT16,
           "uint16": _lib.ISO_UINT16, "int32": _lib.ISO_INT32, "float64": _lib.ISO_FLOAT64}


def _dtype_code(dtype):
    """iso_dtype of a numpy or torch dtype (the VTK scalar types the reference reads, plus uint8)."""
    name = str(dtype).replace("torch.", "")
    if name not in _DTYPES:
        raise ValueError("unsupported sample type %s" % (dtype,))
    return _DTYPES[name]


def make_grid(dims, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
    g = IsoGrid()
    for a in range(3):
        g.dims[a] = int(dims[a])
        g.spacing[a] = float(spacing[a])
        g.origin[a] = float(origin[a])
    return g


class Context:
    """An iso_ctx: one device, its case tables and reusable scratch."""

    def __init__(self, device=0):
        lib = load()
        h = C.c_void_p()
        check(lib.iso_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            load().iso_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scratch_bytes(self):
        return int(load().iso_ctx_scratch_bytes(self.handle))


_DEFAULT = {}


def default_context(device=0):
    ctx = _DEFAULT.get(device)
    if ctx is None:
        ctx = _DEFAULT[device] = Context(device)
    return ctx


class Image3D:
    """Volume on the host: float32 values x fastest, spacing, zero position."""

    def __init__(self, data, spacing, zeroPos, dimensions):
        dims = [int(d) for d in dimensions]
        arr = np.ascontiguousarray(np.asarray(data, dtype=np.float32).reshape(-1))
        if arr.size != dims[0] * dims[1] * dims[2]:
            raise ValueError("data has %d values, dimensions %s need %d" % (arr.size, dims, np.prod(dims)))
        self.data = arr
        # scalar_t is float (FlyingEdges_Config.h:22): keep float32 values
        self.spacing = tuple(float(np.float32(s)) for s in spacing)
        self.zeroPos = tuple(float(np.float32(z)) for z in zeroPos)
        self.dims = tuple(dims)

    @classmethod
    def from_array(cls, vol, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
        """vol indexed [k][j][i] (z, y, x)."""
        nz, ny, nx = vol.shape
        return cls(vol.reshape(-1), spacing, origin, (nx, ny, nz))

    def xdimension(self):
        return self.dims[0]

    def ydimension(self):
        return self.dims[1]

    def zdimension(self):
        return self.dims[2]

    def getSpacing(self):
        return self.spacing

    def getZeroPos(self):
        return self.zeroPos

    def pointer(self):
        return self.data

    def grid(self):
        return make_grid(self.dims, self.spacing, self.zeroPos)

    def array(self):
        return self.data.reshape(self.dims[2], self.dims[1], self.dims[0])


class TriangleMesh:
    """points / normals (V, 3) float32 and triangles (T, 3) vertex indices."""

    def __init__(self, points, normals, triangles):
        self.points = points
        self.normals = normals
        self.triangles = triangles

    def numberOfVertices(self):
        return int(self.points.shape[0])

    def numberOfTriangles(self):
        return int(self.triangles.shape[0])


def _host_mesh_buffers(nv, nt, index_bytes):
    pts = np.empty((max(nv, 1), 3), np.float32)
    nrm = np.empty((max(nv, 1), 3), np.float32)
    tri = np.empty((max(nt, 1), 3), np.uint64 if index_bytes == 8 else np.uint32)
    m = IsoMesh()
    m.points, m.normals, m.tris = pts.ctypes.data, nrm.ctypes.data, tri.ctypes.data
    m.index_bytes = index_bytes
    m.cap_points, m.cap_tris = nv, nt
    return m, pts, nrm, tri


def extract(image, isoval, algorithm=FLYING_EDGES, index_bytes=8, ctx=None):
    """One extraction, host volume in, host TriangleMesh out (iso_extract_host)."""
    lib = load()
    ctx = ctx or default_context()
    algo = _algo(algorithm)
    g = image.grid()
    nv, nt = 0, 0
    for _ in range(2):
        m, pts, nrm, tri = _host_mesh_buffers(nv, nt, index_bytes)
        st = lib.iso_extract_host(ctx.handle, algo, _ptr(image.data), C.byref(g), C.c_float(isoval),
                                  C.byref(m), None)
        if st == _lib.ISO_ERR_CAPACITY:
            nv, nt = m.n_points, m.n_tris
            continue
        check(st, ctx.handle)
        return TriangleMesh(pts[: m.n_points], nrm[: m.n_points], tri[: m.n_tris])
    raise RuntimeError("output size changed between two extractions of the same volume")


def extract_typed(volume, isoval, algorithm=FLYING_EDGES, spacing=(1, 1, 1), origin=(0, 0, 0), index_bytes=8,
                  ctx=None):
    """Host array of any supported sample type ([k][j][i]) in, TriangleMesh out:
    the samples cross to the device as they are and become float32 there
    (iso_extract_host_typed); the mesh equals extracting volume.astype(float32)."""
    lib = load()
    ctx = ctx or default_context()
    algo = _algo(algorithm)
    vol = np.ascontiguousarray(volume)
    dcode = _dtype_code(vol.dtype)
    g = make_grid((vol.shape[2], vol.shape[1], vol.shape[0]), spacing, origin)
    nv, nt = 0, 0
    for _ in range(2):
        m, pts, nrm, tri = _host_mesh_buffers(nv, nt, index_bytes)
        st = lib.iso_extract_host_typed(ctx.handle, algo, _ptr(vol), dcode, C.byref(g), C.c_float(isoval), C.byref(m),
                                        None)
        if st == _lib.ISO_ERR_CAPACITY:
            nv, nt = m.n_points, m.n_tris
            continue
        check(st, ctx.handle)
        return TriangleMesh(pts[: m.n_points], nrm[: m.n_points], tri[: m.n_tris])
    raise RuntimeError("output size changed between two extractions of the same volume")


def MarchingCubes(image, isoval, ctx=None):
    """marchingCubes/serial/main.cpp:42-192: mesh with MC vertex numbering."""
    return extract(image, isoval, MARCHING_CUBES, 8, ctx)


class FlyingEdgesAlgorithm:
    """flyingEdges/serial/FlyingEdgesAlgorithm.h:29-49, backed by the GPU passes."""

    def __init__(self, image, isoval, ctx=None):
        lib = load()
        self._ctx = ctx or default_context()
        self._image = image  # the reference keeps a reference to the image too
        self._grid = image.grid()
        self.isoval = float(isoval)
        h = C.c_void_p()
        check(lib.iso_fe_create(self._ctx.handle, _ptr(image.data), C.byref(self._grid), C.c_float(isoval),
                                C.byref(h)), self._ctx.handle)
        self._h = h

    def __del__(self):
        try:
            if self._h:
                load().iso_fe_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def _call(self, fn):
        check(fn(self._h), self._ctx.handle)

    def pass1(self):
        self._call(load().iso_fe_pass1)

    def pass2(self):
        self._call(load().iso_fe_pass2)

    def pass3(self):
        self._call(load().iso_fe_pass3)

    def pass4(self):
        self._call(load().iso_fe_pass4)

    def sizes(self):
        nv, nt = C.c_int64(), C.c_int64()
        check(load().iso_fe_sizes(self._h, C.byref(nv), C.byref(nt)), self._ctx.handle)
        return nv.value, nt.value

    def gridEdges(self):
        """(ny*nz, 5) records {xl, xr, xstart, ystart, zstart} and triCounter."""
        nx, ny, nz = self._image.dims
        ge = np.zeros((ny * nz, 5), np.uint64)
        tc = np.zeros(max((ny - 1) * (nz - 1), 1), np.uint64)
        check(load().iso_fe_grid_edges(self._h, ge.ctypes.data, tc.ctypes.data), self._ctx.handle)
        return ge, tc[: (ny - 1) * (nz - 1)]

    def moveOutput(self, index_bytes=8):
        nv, nt = self.sizes()
        m, pts, nrm, tri = _host_mesh_buffers(nv, nt, index_bytes)
        check(load().iso_fe_move_output(self._h, C.byref(m)), self._ctx.handle)
        return TriangleMesh(pts[:nv], nrm[:nv], tri[:nt])


class DeviceMesh:
    """Mesh in device memory (torch tensors with spare capacity)."""

    def __init__(self, cap_points, cap_tris, index_bytes=4, device="cuda"):
        import torch
        self.index_bytes = index_bytes
        self.points = torch.empty((max(cap_points, 1), 3), dtype=torch.float32, device=device)
        self.normals = torch.empty((max(cap_points, 1), 3), dtype=torch.float32, device=device)
        self.tris = torch.empty((max(cap_tris, 1), 3), dtype=torch.int32 if index_bytes == 4 else torch.int64,
                                device=device)
        self.n_points = 0
        self.n_tris = 0

    def descriptor(self):
        m = IsoMesh()
        m.points, m.normals, m.tris = _ptr(self.points), _ptr(self.normals), _ptr(self.tris)
        m.index_bytes = self.index_bytes
        m.cap_points = self.points.shape[0]
        m.cap_tris = self.tris.shape[0]
        return m


def extract_device(volume, dims, isoval, algorithm=FLYING_EDGES, spacing=(1, 1, 1), origin=(0, 0, 0),
                   out=None, index_bytes=4, ctx=None, stream=None):
    """Extraction of a device-resident volume (a CUDA float32 tensor, x fastest).

    Returns a DeviceMesh; `out` is reused when its capacity suffices and is
    re-allocated (exact size) otherwise.
    """
    import torch
    lib = load()
    ctx = ctx or default_context(volume.device.index or 0)
    algo = _algo(algorithm)
    g = make_grid(dims, spacing, origin)
    if not volume.is_cuda or not volume.is_contiguous():
        raise ValueError("volume must be a contiguous CUDA tensor")
    dcode = _dtype_code(volume.dtype)  # narrow types are converted to float32 on the device
    s = stream if stream is not None else torch.cuda.current_stream(volume.device).cuda_stream
    if out is None:
        out = DeviceMesh(0, 0, index_bytes, volume.device)
    for _ in range(2):
        m = out.descriptor()
        if dcode == _lib.ISO_FLOAT32:
            st = lib.iso_extract_device(ctx.handle, algo, _ptr(volume), C.byref(g), C.c_float(isoval), C.byref(m),
                                        C.c_void_p(s))
        else:
            st = lib.iso_extract_device_typed(ctx.handle, algo, _ptr(volume), dcode, C.byref(g), C.c_float(isoval),
                                              C.byref(m), C.c_void_p(s))
        if st == _lib.ISO_ERR_CAPACITY:
            out = DeviceMesh(m.n_points, m.n_tris, out.index_bytes, volume.device)
            continue
        check(st, ctx.handle)
        out.n_points, out.n_tris = m.n_points, m.n_tris
        return out
    raise RuntimeError("output size changed between two extractions of the same volume")


class Request:
    """One extraction of a batch: a contiguous CUDA float32 volume (x fastest)
    with its grid, isovalue and algorithm."""

    def __init__(self, volume, dims, isoval, algorithm=FLYING_EDGES, spacing=(1, 1, 1), origin=(0, 0, 0)):
        if not volume.is_cuda or not volume.is_contiguous() or str(volume.dtype) != "torch.float32":
            raise ValueError("a batch volume must be a contiguous CUDA float32 tensor")
        self.volume = volume
        self.dims = tuple(int(d) for d in dims)
        self.isoval = float(isoval)
        self.algorithm = algorithm
        self.spacing = spacing
        self.origin = origin
        self._desc = None

    def descriptor(self):
        """The iso_request of this request (built once; copies of it go into the C arrays)."""
        if self._desc is None:
            r = _lib.IsoRequest()
            r.volume = _ptr(self.volume)
            r.grid = make_grid(self.dims, self.spacing, self.origin)
            r.isoval = self.isoval
            r.algorithm = _algo(self.algorithm)
            self._desc = r
        return self._desc


class Batch:
    """Requests and their meshes as the C arrays of iso_extract_batch, built
    once: running the same Batch again relaunches the captured graph."""

    def __init__(self, requests, meshes):
        self.requests = list(requests)
        self.meshes = list(meshes)
        n = len(self.requests)
        self.req = (_lib.IsoRequest * max(n, 1))(*[r.descriptor() for r in self.requests])
        self.out = (IsoMesh * max(n, 1))(*[m.descriptor() for m in self.meshes])
        self.status = (C.c_int * max(n, 1))()

    def run(self, ctx=None, stream=None):
        """One iso_extract_batch call; returns the per-request statuses."""
        import torch
        lib = load()
        ctx = ctx or default_context()
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        n = len(self.requests)
        st = lib.iso_extract_batch(ctx.handle, n, self.req, self.out, self.status, C.c_void_p(s))
        for i, m in enumerate(self.meshes):
            m.n_points, m.n_tris = self.out[i].n_points, self.out[i].n_tris
        codes = [self.status[i] for i in range(n)]
        if st not in (_lib.ISO_OK, _lib.ISO_ERR_CAPACITY) or any(
                c not in (_lib.ISO_OK, _lib.ISO_ERR_CAPACITY) for c in codes):
            check(st if st != _lib.ISO_OK else next(c for c in codes if c != _lib.ISO_OK), ctx.handle)
        return codes


class PackedBuffers:
    """Device buffers of packed batches (iso_extract_batch_packed), reused from batch to batch and grown
    (a quarter more than asked) when a batch needs more."""

    def __init__(self, cap_points=0, cap_tris=0, index_bytes=4, device="cuda"):
        self.index_bytes = index_bytes
        self.device = device
        self.points = self.normals = self.tris = None
        self.reserve(cap_points, cap_tris)

    def reserve(self, cap_points, cap_tris):
        import torch
        have_p = self.points.shape[0] if self.points is not None else 0
        have_t = self.tris.shape[0] if self.tris is not None else 0
        if cap_points > have_p or self.points is None:
            n = max(cap_points + cap_points // 4, 1)
            self.points = self.normals = None
            self.points = torch.empty((n, 3), dtype=torch.float32, device=self.device)
            self.normals = torch.empty((n, 3), dtype=torch.float32, device=self.device)
        if cap_tris > have_t or self.tris is None:
            n = max(cap_tris + cap_tris // 4, 1)
            self.tris = None
            self.tris = torch.empty((n, 3), dtype=torch.int32 if self.index_bytes == 4 else torch.int64,
                                    device=self.device)


class PackedMesh:
    """One request's mesh inside a packed batch's buffers: its offsets and counts, with the DeviceMesh views
    (points, normals, tris) made when they are read."""

    __slots__ = ("buffers", "point_first", "tri_first", "n_points", "n_tris", "index_bytes")

    def __init__(self, buffers, point_first, tri_first, n_points, n_tris):
        self.buffers = buffers
        self.point_first, self.tri_first = point_first, tri_first
        self.n_points, self.n_tris = n_points, n_tris
        self.index_bytes = buffers.index_bytes

    @property
    def points(self):
        return self.buffers.points[self.point_first: self.point_first + max(self.n_points, 1)]

    @property
    def normals(self):
        return self.buffers.normals[self.point_first: self.point_first + max(self.n_points, 1)]

    @property
    def tris(self):
        return self.buffers.tris[self.tri_first: self.tri_first + max(self.n_tris, 1)]


def extract_batch_packed(requests, buffers=None, index_bytes=4, ctx=None, stream=None):
    """Batched extraction into one set of buffers (iso_extract_batch_packed): a list of Request (Flying Edges,
    rows of at most 512 points) in, one PackedMesh per request out (points, normals and tris views into
    `buffers`, a PackedBuffers made or grown as needed) holding what extract_device gives for its request.
    Returns (meshes, buffers).  A batch that does not fit grows the buffers to its total and runs again."""
    import torch
    lib = load()
    requests = list(requests)
    n = len(requests)
    if buffers is None:
        buffers = PackedBuffers(0, 0, index_bytes, requests[0].volume.device if requests else "cuda")
    ctx = ctx or default_context()
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    req = (_lib.IsoRequest * max(n, 1))(*[r.descriptor() for r in requests])
    pf, tf, nv, nt = [(C.c_int64 * max(n, 1))() for _ in range(4)]
    status = (C.c_int * max(n, 1))()
    for _ in range(2):
        st = lib.iso_extract_batch_packed(ctx.handle, n, req, _ptr(buffers.points), _ptr(buffers.normals),
                                          _ptr(buffers.tris), buffers.index_bytes, buffers.points.shape[0],
                                          buffers.tris.shape[0], pf, tf, nv, nt, status, C.c_void_p(s))
        if st != _lib.ISO_ERR_CAPACITY:
            break
        buffers.reserve(sum(nv[i] for i in range(n)), sum(nt[i] for i in range(n)))
    check(st, ctx.handle)
    return [PackedMesh(buffers, pf[i], tf[i], nv[i], nt[i]) for i in range(n)], buffers


def extract_batch(requests, meshes=None, index_bytes=4, ctx=None, stream=None, predictor=None):
    """Batched extraction (iso_extract_batch): a list of Request in, a list
    of DeviceMesh out, each what extract_device gives for its request.

    Meshes too small for their request (or none given) come back with the
    sizes needed from the first batch run; they are re-allocated at exactly
    that size and those requests run again as one more batch.  With a
    predictor (predictor.Predictor) and no meshes, the meshes are sized by the
    output-size network first (one launch for the whole batch), so most
    requests run once.
    """
    requests = list(requests)
    if meshes is None and predictor is not None and requests:
        from .predictor import block_stats
        stats = {}
        for r in requests:  # each distinct volume's block statistics once
            key = (r.volume.data_ptr(), r.dims)
            if key not in stats:
                stats[key] = block_stats(r.volume, r.dims, stream)
        caps = predictor.capacities([(stats[(r.volume.data_ptr(), r.dims)], r.isoval) for r in requests], stream)
        meshes = [DeviceMesh(v, t, index_bytes, r.volume.device) for (v, t), r in zip(caps, requests)]
    if meshes is None:
        meshes = [DeviceMesh(0, 0, index_bytes, r.volume.device) for r in requests]
    meshes = list(meshes)
    codes = Batch(requests, meshes).run(ctx, stream)
    redo = [i for i, c in enumerate(codes) if c == _lib.ISO_ERR_CAPACITY]
    if redo:
        for i in redo:
            meshes[i] = DeviceMesh(meshes[i].n_points, meshes[i].n_tris, meshes[i].index_bytes,
                                   requests[i].volume.device)
        codes = Batch([requests[i] for i in redo], [meshes[i] for i in redo]).run(ctx, stream)
        if any(c != _lib.ISO_OK for c in codes):
            raise RuntimeError("output size changed between two extractions of the same volume")
    return meshes


def set_batch_lanes(lanes, ctx=None):
    """Lanes of the batched path (0: the autotuner picks them on the next batch)."""
    ctx = ctx or default_context()
    check(load().iso_batch_set_lanes(ctx.handle, int(lanes)), ctx.handle)


def set_graph(enable, ctx=None):
    """Graph mode of the one-shot device extraction (iso_ctx_set_graph): repeated calls relaunch a
    captured CUDA graph."""
    ctx = ctx or default_context()
    check(load().iso_ctx_set_graph(ctx.handle, 1 if enable else 0), ctx.handle)


def set_batch_graph(enable, ctx=None):
    """Capture batches as CUDA graphs (default) or launch their lanes directly."""
    ctx = ctx or default_context()
    check(load().iso_batch_set_graph(ctx.handle, 1 if enable else 0), ctx.handle)


def set_batch_fused(mode, ctx=None):
    """How a batch runs its Flying Edges requests of rows up to 512 points (iso_batch_set_fused): False / 0 on the
    lanes, True / 1 (default) one launch per pass when at least 16 of them, 2 always one launch per pass."""
    ctx = ctx or default_context()
    check(load().iso_batch_set_fused(ctx.handle, int(mode)), ctx.handle)


def batch_fused_split(ctx=None):
    """(count planes, items per warp) of the fused launches as the autotuner chose them ((0, 0) before)."""
    ctx = ctx or default_context()
    kc, ipw = C.c_int(), C.c_int()
    check(load().iso_batch_fused_split(ctx.handle, C.byref(kc), C.byref(ipw)), ctx.handle)
    return kc.value, ipw.value


def batch_lanes(ctx=None):
    ctx = ctx or default_context()
    return int(load().iso_batch_lanes(ctx.handle))


def set_batch_split(share, ctx=None):
    """Work split of the batched path: plans sized for nsm / share SMs (0: the autotuner picks it)."""
    ctx = ctx or default_context()
    check(load().iso_batch_set_split(ctx.handle, int(share)), ctx.handle)


def batch_split(ctx=None):
    ctx = ctx or default_context()
    return int(load().iso_batch_split(ctx.handle))


def count_device(volume, dims, isoval, algorithm=FLYING_EDGES, ctx=None, stream=None):
    """Passes 1-3 only: exact (n_points, n_tris) of a device-resident volume."""
    import torch
    lib = load()
    ctx = ctx or default_context(volume.device.index or 0)
    g = make_grid(dims)
    s = stream if stream is not None else torch.cuda.current_stream(volume.device).cuda_stream
    nv, nt = C.c_int64(), C.c_int64()
    check(lib.iso_count_device(ctx.handle, _algo(algorithm), _ptr(volume), C.byref(g), C.c_float(isoval),
                               C.byref(nv), C.byref(nt), C.c_void_p(s)), ctx.handle)
    return nv.value, nt.value


# ---------------------------------------------------------------------------
# VTK IO and synthetic volumes
# ---------------------------------------------------------------------------
def _io_check(st, path):
    if st == _lib.ISO_ERR_IO:
        raise file_not_found(path)
    if st == _lib.ISO_ERR_FORMAT:
        raise bad_format(path)
    check(st)


def loadImage(path):
    lib = load()
    g = IsoGrid()
    p = os.fsencode(path)
    _io_check(lib.iso_vtk_read_image(p, C.byref(g), None), path)
    dims = [g.dims[a] for a in range(3)]
    data = np.empty(int(np.prod(dims)), np.float32)
    _io_check(lib.iso_vtk_read_image(p, C.byref(g), data.ctypes.data), path)
    return Image3D(data, list(g.spacing), list(g.origin), dims)


def saveImage(image, path):
    g = image.grid()
    _io_check(load().iso_vtk_write_image(os.fsencode(path), C.byref(g), image.data.ctypes.data), path)


def saveTriangleMesh(mesh, path):
    pts = np.ascontiguousarray(mesh.points, np.float32)
    nrm = np.ascontiguousarray(mesh.normals, np.float32)
    tri = np.ascontiguousarray(mesh.triangles)
    m = IsoMesh()
    m.points, m.normals, m.tris = pts.ctypes.data, nrm.ctypes.data, tri.ctypes.data
    m.index_bytes = tri.dtype.itemsize
    m.n_points, m.n_tris = pts.shape[0], tri.shape[0]
    m.cap_points, m.cap_tris = m.n_points, m.n_tris
    _io_check(load().iso_vtk_write_mesh(os.fsencode(path), C.byref(m)), path)


def generate_blobs(dims, nblobs=8, seed=0):
    """[k][j][i] float32 array: sum of nblobs Gaussian blobs."""
    d = (C.c_int64 * 3)(*[int(x) for x in dims])
    out = np.empty((dims[2], dims[1], dims[0]), np.float32)
    check(load().iso_generate_blobs(d, int(nblobs), C.c_uint64(seed), out.ctypes.data))
    return out


def generate_value_noise(dims, octaves=4, period=64, seed=0):
    """[k][j][i] float32 array: octave value noise in about [-2, 2]."""
    d = (C.c_int64 * 3)(*[int(x) for x in dims])
    out = np.empty((dims[2], dims[1], dims[0]), np.float32)
    check(load().iso_generate_value_noise(d, int(octaves), int(period), C.c_uint64(seed), out.ctypes.data))
    return out
