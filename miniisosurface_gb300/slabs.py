"""z-slab decomposition: sharding over GPUs and streaming large volumes.

The grid's planes are split into slabs [k0, k1).  A slab owns the Flying Edges
vertices of the grid rows of its planes, the cells between planes k0 and k1
and, for Marching Cubes, the vertices those cells own, so the global vertex
and triangle order (row order for FE, owner-cell order for MC) is the
concatenation of the slabs' parts.  Each slab reads planes k0-1 .. k1+1 (the
gradient halo; marchingCubes/mpi/mpiutil.h:197-203 reads DataBeg = Beg-1 ..
DataEnd = End+2 the same way) and needs one exchange: an exclusive scan of
the slabs' (vertex, triangle) counts, which gives each slab its first vertex
id and first triangle index.  No mesh is merged.

  partition(nz, n)          n slabs of about equal plane counts
  data_planes(k0, k1, nz)   planes a slab reads
  exclusive_offsets(counts) the count exchange on one host
  exchange_counts(...)      the same over torch.distributed ranks (all-gather of two integers per rank)
  count_slab / extract_slab the C ABI calls (iso_count_slab, iso_extract_slab)
  extract_multislab         single-GPU multi-slab extraction: every slab in turn into one mesh
"""
import ctypes as C

from . import _lib
from ._lib import check, load
from .api import DeviceMesh, _algo, _ptr, default_context, make_grid


def partition(nz, n):
    """n contiguous slabs [k0, k1) of the planes 0 .. nz-1 (n is capped at nz)."""
    n = max(1, min(int(n), int(nz)))
    bounds = [round(i * nz / n) for i in range(n + 1)]
    return [(bounds[i], bounds[i + 1]) for i in range(n)]


def data_planes(k0, k1, nz):
    """First and last plane a slab reads: max(k0-1, 0) .. min(k1+1, nz-1)."""
    return max(k0 - 1, 0), min(k1 + 1, nz - 1)


def exclusive_offsets(counts):
    """[(V, T) per slab] -> [(first vertex id, first triangle index) per slab], totals."""
    offs, v, t = [], 0, 0
    for cv, ct in counts:
        offs.append((v, t))
        v += int(cv)
        t += int(ct)
    return offs, (v, t)


def exchange_counts(n_points, n_tris, group=None):
    """The slabs' count exchange over torch.distributed: every rank holds one
    slab, in rank order.  Returns (point_offset, tri_offset) of this rank and
    the totals.  Works with the gloo and NCCL backends (two int64 per rank)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    mine = torch.tensor([int(n_points), int(n_tris)], dtype=torch.int64, device=dev)
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    counts = [tuple(int(x) for x in p.cpu()) for p in parts]
    offs, totals = exclusive_offsets(counts)
    return offs[dist.get_rank(group)], totals


def _window(volume, dims, k0, k1):
    """The planes a slab reads, as a view of a whole-volume device tensor."""
    nx, ny, nz = (int(d) for d in dims)
    d0, d1 = data_planes(k0, k1, nz)
    plane = nx * ny
    return volume[d0 * plane:(d1 + 1) * plane]


def count_slab(window, dims, k0, k1, isoval, algorithm, spacing=(1, 1, 1), origin=(0, 0, 0), ctx=None,
               stream=None):
    """Vertex and triangle counts of slab [k0, k1); window holds its data planes."""
    import torch

    lib = load()
    ctx = ctx or default_context(window.device.index or 0)
    g = make_grid(dims, spacing, origin)
    s = stream if stream is not None else torch.cuda.current_stream(window.device).cuda_stream
    nv, nt = C.c_int64(), C.c_int64()
    check(lib.iso_count_slab(ctx.handle, _algo(algorithm), _ptr(window), C.byref(g), int(k0), int(k1),
                             C.c_float(isoval), C.byref(nv), C.byref(nt), C.c_void_p(s)), ctx.handle)
    return nv.value, nt.value


def extract_slab(window, dims, k0, k1, isoval, algorithm, point_offset, tri_offset, out, spacing=(1, 1, 1),
                 origin=(0, 0, 0), ctx=None, stream=None):
    """Slab [k0, k1) into `out` (a DeviceMesh, or any object with a descriptor()
    of the slab's rows): vertices from id point_offset, triangles from index
    tri_offset."""
    import torch

    lib = load()
    ctx = ctx or default_context(window.device.index or 0)
    g = make_grid(dims, spacing, origin)
    s = stream if stream is not None else torch.cuda.current_stream(window.device).cuda_stream
    m = out.descriptor()
    check(lib.iso_extract_slab(ctx.handle, _algo(algorithm), _ptr(window), C.byref(g), int(k0), int(k1),
                               C.c_float(isoval), int(point_offset), int(tri_offset), C.byref(m), C.c_void_p(s)),
          ctx.handle)
    return m.n_points, m.n_tris


class _SlabView:
    """Rows [v0, v0+nv) / [t0, t0+nt) of a DeviceMesh as an iso_mesh."""

    def __init__(self, mesh, v0, nv, t0, nt):
        self.mesh, self.v0, self.nv, self.t0, self.nt = mesh, v0, nv, t0, nt

    def descriptor(self):
        m = _lib.IsoMesh()
        mesh = self.mesh
        m.points = _ptr(mesh.points) + 12 * self.v0
        m.normals = _ptr(mesh.normals) + 12 * self.v0
        m.tris = _ptr(mesh.tris) + 3 * mesh.index_bytes * self.t0
        m.index_bytes = mesh.index_bytes
        m.cap_points = self.nv
        m.cap_tris = self.nt
        return m


def extract_multislab(volume, dims, isoval, algorithm, nslabs, spacing=(1, 1, 1), origin=(0, 0, 0),
                      index_bytes=4, ctx=None, stream=None):
    """Single-GPU multi-slab extraction: counts of every slab, the exchange
    (an exclusive scan here), then every slab into its part of one mesh.
    The result equals extract_device on the whole volume."""
    nz = int(dims[2])
    slabs = partition(nz, nslabs)
    counts = [count_slab(_window(volume, dims, k0, k1), dims, k0, k1, isoval, algorithm, spacing, origin, ctx,
                         stream) for k0, k1 in slabs]
    offs, (V, T) = exclusive_offsets(counts)
    mesh = DeviceMesh(V, T, index_bytes, volume.device)
    for (k0, k1), (v0, t0), (nv, nt) in zip(slabs, offs, counts):
        got = extract_slab(_window(volume, dims, k0, k1), dims, k0, k1, isoval, algorithm, v0, t0,
                           _SlabView(mesh, v0, nv, t0, nt), spacing, origin, ctx, stream)
        if got != (nv, nt):
            raise RuntimeError("slab [%d, %d) changed size between count and extraction" % (k0, k1))
    mesh.n_points, mesh.n_tris = V, T
    return mesh
