"""Test infrastructure: ctypes wrapper of the C oracle (oracle/liboracle.so)
and helpers that run the reference binaries built by oracle/build_ref.sh.

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "lib" / "liboracle.so"
REF_DIR = ORACLE_DIR / "_ref"
# the miniIsosurface checkout read by the tests that compare with its sources (MINIISO_REFERENCE)
REFERENCE = Path(os.environ.get("MINIISO_REFERENCE", "/root/reference"))


class OracleMesh(C.Structure):
    _fields_ = [("n_points", C.c_size_t), ("n_tris", C.c_size_t), ("points", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("tris", C.POINTER(C.c_size_t)),
                ("edge_of_vertex", C.POINTER(C.c_size_t))]


_LIB = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)


def lib():
    global _LIB
    if _LIB is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        L = C.CDLL(str(ORACLE_LIB))
        sz3 = C.c_size_t * 3
        f3 = C.c_float * 3
        L.oracle_fe_run.argtypes = [C.c_void_p, sz3, f3, f3, C.c_float, C.c_int, C.POINTER(OracleMesh)]
        L.oracle_mc_run.argtypes = [C.c_void_p, sz3, f3, f3, C.c_float, C.POINTER(OracleMesh)]
        L.oracle_mc_dupfree_run.argtypes = [C.c_void_p, sz3, f3, f3, C.c_float, C.POINTER(OracleMesh)]
        L.oracle_mc_openmp_run.argtypes = [C.c_void_p, sz3, f3, f3, C.c_float, C.c_int, C.POINTER(OracleMesh)]
        L.oracle_generate_blobs.argtypes = [sz3, C.c_int, C.c_uint64, C.c_void_p]
        L.oracle_generate_value_noise.argtypes = [sz3, C.c_int, C.c_int, C.c_uint64, C.c_void_p]
        L.oracle_mesh_free.argtypes = [C.POINTER(OracleMesh)]
        L.oracle_fe_create.restype = C.c_void_p
        L.oracle_fe_create.argtypes = [C.c_void_p, sz3, f3, f3, C.c_float, C.c_int]
        for n in ("oracle_fe_pass1", "oracle_fe_pass2", "oracle_fe_pass3", "oracle_fe_pass4", "oracle_fe_destroy"):
            getattr(L, n).argtypes = [C.c_void_p]
        L.oracle_fe_grid_edges.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_fe_tri_counter.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_fe_take.argtypes = [C.c_void_p, C.POINTER(OracleMesh)]
        L.oracle_block_tris.argtypes = [C.c_void_p, sz3, C.c_float, C.c_int, C.c_void_p]
        L.oracle_last_wall_seconds.restype = C.c_double
        L.oracle_mc_last_wall_seconds.restype = C.c_double
        _LIB = L
    return _LIB


def _mesh_to_numpy(m):
    nv, nt = m.n_points, m.n_tris
    pts = np.ctypeslib.as_array(m.points, (max(3 * nv, 1),))[: 3 * nv].reshape(nv, 3).copy()
    nrm = np.ctypeslib.as_array(m.normals, (max(3 * nv, 1),))[: 3 * nv].reshape(nv, 3).copy()
    tri = np.ctypeslib.as_array(m.tris, (max(3 * nt, 1),))[: 3 * nt].reshape(nt, 3).astype(np.uint64)
    eov = np.ctypeslib.as_array(m.edge_of_vertex, (max(nv, 1),))[:nv].astype(np.uint64)
    return pts, nrm, tri, eov


def _args(vol, spacing, origin):
    vol = np.ascontiguousarray(vol, np.float32)
    nz, ny, nx = vol.shape
    dims = (C.c_size_t * 3)(nx, ny, nz)
    sp = (C.c_float * 3)(*spacing)
    org = (C.c_float * 3)(*origin)
    return vol, dims, sp, org


def fe(vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0), nthreads=1):
    """Oracle Flying Edges of vol[k][j][i]: (points, normals, tris, edge_of_vertex)."""
    L = lib()
    vol, dims, sp, org = _args(vol, spacing, origin)
    m = OracleMesh()
    if any(d < 2 for d in vol.shape):
        return (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint64),
                np.zeros(0, np.uint64))
    L.oracle_fe_run(vol.ctypes.data, dims, sp, org, C.c_float(iso), int(nthreads), C.byref(m))
    try:
        return _mesh_to_numpy(m)
    finally:
        L.oracle_mesh_free(C.byref(m))


def block_tris(vol, iso, block=16):
    """Triangles per block of block^3 cells (oracle_block_tris)."""
    vol = np.ascontiguousarray(vol, dtype=np.float32)
    nz, ny, nx = vol.shape
    nb = [max(0, (n - 2) // block + 1) if n >= 2 else 0 for n in (nx, ny, nz)]
    out = np.zeros(nb[0] * nb[1] * nb[2], dtype=np.int32)
    if out.size:
        dims = (C.c_size_t * 3)(nx, ny, nz)
        lib().oracle_block_tris(vol.ctypes.data, dims, C.c_float(iso), block, out.ctypes.data)
    return out


def fe_wall_seconds():
    return lib().oracle_last_wall_seconds()


def mc_wall_seconds():
    return lib().oracle_mc_last_wall_seconds()


def mc(vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0)):
    L = lib()
    vol, dims, sp, org = _args(vol, spacing, origin)
    if any(d < 2 for d in vol.shape):
        return (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint64),
                np.zeros(0, np.uint64))
    m = OracleMesh()
    L.oracle_mc_run(vol.ctypes.data, dims, sp, org, C.c_float(iso), C.byref(m))
    try:
        return _mesh_to_numpy(m)
    finally:
        L.oracle_mesh_free(C.byref(m))


def mc_openmp(vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0), nthreads=1):
    """Oracle port of marchingCubes/openmp: nthreads z-sections, seam vertices once per section."""
    L = lib()
    vol, dims, sp, org = _args(vol, spacing, origin)
    if any(d < 2 for d in vol.shape):
        return (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint64),
                np.zeros(0, np.uint64))
    m = OracleMesh()
    L.oracle_mc_openmp_run(vol.ctypes.data, dims, sp, org, C.c_float(iso), int(nthreads), C.byref(m))
    try:
        return _mesh_to_numpy(m)
    finally:
        L.oracle_mesh_free(C.byref(m))


def generate_blobs(dims, nblobs=8, seed=0):
    """The seeded Gaussian-blob volume (oracle/volgen_oracle.c), shape (nz, ny, nx)."""
    nx, ny, nz = (int(d) for d in dims)
    out = np.empty((nz, ny, nx), np.float32)
    if lib().oracle_generate_blobs((C.c_size_t * 3)(nx, ny, nz), int(nblobs), C.c_uint64(seed), out.ctypes.data):
        raise ValueError("oracle_generate_blobs failed")
    return out


def generate_value_noise(dims, octaves=4, period=64, seed=0):
    """The seeded value-noise volume (oracle/volgen_oracle.c), shape (nz, ny, nx)."""
    nx, ny, nz = (int(d) for d in dims)
    out = np.empty((nz, ny, nx), np.float32)
    if lib().oracle_generate_value_noise((C.c_size_t * 3)(nx, ny, nz), int(octaves), int(period), C.c_uint64(seed),
                                         out.ctypes.data):
        raise ValueError("oracle_generate_value_noise failed")
    return out


def mc_dupfree(vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0)):
    """Oracle MC with vertices in global-edge-index order (marchingCubes/openmpDupFree, one thread)."""
    L = lib()
    vol, dims, sp, org = _args(vol, spacing, origin)
    if any(d < 2 for d in vol.shape):
        return (np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint64),
                np.zeros(0, np.uint64))
    m = OracleMesh()
    L.oracle_mc_dupfree_run(vol.ctypes.data, dims, sp, org, C.c_float(iso), C.byref(m))
    try:
        return _mesh_to_numpy(m)
    finally:
        L.oracle_mesh_free(C.byref(m))


def fe_passes(vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0)):
    """Oracle intermediate state: gridEdges and triCounter after pass 2 and 3."""
    L = lib()
    vol, dims, sp, org = _args(vol, spacing, origin)
    nz, ny, nx = vol.shape
    h = L.oracle_fe_create(vol.ctypes.data, dims, sp, org, C.c_float(iso), 1)
    try:
        L.oracle_fe_pass1(h)
        L.oracle_fe_pass2(h)
        ge2 = np.zeros((ny * nz, 5), np.uint64)
        tc2 = np.zeros(max((ny - 1) * (nz - 1), 1), np.uint64)
        L.oracle_fe_grid_edges(h, ge2.ctypes.data)
        L.oracle_fe_tri_counter(h, tc2.ctypes.data)
        L.oracle_fe_pass3(h)
        ge3 = np.zeros((ny * nz, 5), np.uint64)
        tc3 = np.zeros(max((ny - 1) * (nz - 1), 1), np.uint64)
        L.oracle_fe_grid_edges(h, ge3.ctypes.data)
        L.oracle_fe_tri_counter(h, tc3.ctypes.data)
    finally:
        L.oracle_fe_destroy(h)
    n = (ny - 1) * (nz - 1)
    return ge2, tc2[:n], ge3, tc3[:n]


# ---------------------------------------------------------------------------
# VTK files in the reference layouts (numpy, independent of the product IO)
# ---------------------------------------------------------------------------
def write_structured_points(path, vol, spacing=(1, 1, 1), origin=(0, 0, 0)):
    nz, ny, nx = vol.shape
    with open(path, "wb") as f:
        f.write(b"# vtk DataFile Version 3.0\ntest volume\nBINARY\nDATASET STRUCTURED_POINTS\n")
        f.write(("DIMENSIONS %d %d %d\n" % (nx, ny, nz)).encode())
        f.write(("SPACING %.9g %.9g %.9g\n" % tuple(spacing)).encode())
        f.write(("ORIGIN %.9g %.9g %.9g\n" % tuple(origin)).encode())
        f.write(("POINT_DATA %d\nSCALARS scalars float\nLOOKUP_TABLE default\n" % vol.size).encode())
        f.write(np.ascontiguousarray(vol, ">f4").tobytes())


def read_polydata(path):
    """Reads the mesh layout of util::saveTriangleMesh: (points, normals, tris)."""
    data = Path(path).read_bytes()
    pos = 0

    def line():
        nonlocal pos
        e = data.index(b"\n", pos)
        s = data[pos:e].decode()
        pos = e + 1
        return s

    for _ in range(4):
        line()
    nv = int(line().split()[1])
    pts = np.frombuffer(data, ">f4", 3 * nv, pos).astype(np.float32).reshape(nv, 3)
    pos += 12 * nv
    line()  # end of the points line
    nt = int(line().split()[1])
    recs = np.frombuffer(data, ">u8", 4 * nt, pos).astype(np.uint64).reshape(nt, 4)
    pos += 32 * nt
    line()
    line()  # POINT_DATA
    line()  # NORMALS
    nrm = np.frombuffer(data, ">f4", 3 * nv, pos).astype(np.float32).reshape(nv, 3)
    assert np.all(recs[:, 0] == 3)
    return pts, nrm, recs[:, 1:].copy()


def ref_available(name="flyingEdgesSerial"):
    return (REF_DIR / name).exists()


def run_ref(name, vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0), threads=None):
    """Runs a reference binary on vol and returns (points, normals, tris, yaml text)."""
    with tempfile.TemporaryDirectory() as td:
        vin = os.path.join(td, "in.vtk")
        vout = os.path.join(td, "out.vtk")
        write_structured_points(vin, vol, spacing, origin)
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        res = subprocess.run([str(REF_DIR / name), "-i", vin, "-o", vout, "-v", repr(float(iso)),
                              "-y", os.path.join(td, "run.yaml")], capture_output=True, text=True, env=env,
                             check=True)
        pts, nrm, tri = read_polydata(vout)
        return pts, nrm, tri, res.stdout, Path(vout).read_bytes()


# ---------------------------------------------------------------------------
# FP64 interpolation error of a float32 mesh
# ---------------------------------------------------------------------------
def edge_points(edge_of_vertex, dims):
    """(axis, lower end (i, j, k)) of each vertex from its global edge id
    (marchingCubes/util/Image3D.cpp:168-256: x-edges, then y, then z)."""
    nx, ny, nz = dims
    nX = (nx - 1) * ny * nz
    nY = nx * (ny - 1) * nz
    e = np.asarray(edge_of_vertex).astype(np.int64)
    axis = np.where(e < nX, 0, np.where(e < nX + nY, 1, 2))
    loc = np.where(axis == 0, e, np.where(axis == 1, e - nX, e - nX - nY))
    ex = np.array([nx - 1, nx, nx])[axis]
    ey = np.array([ny, ny - 1, ny])[axis]
    i = loc % ex
    j = (loc // ex) % ey
    k = loc // (ex * ey)
    return axis, np.stack([i, j, k], 1)


def fp64_error(vol, iso, points, normals, edge_of_vertex, spacing=(1, 1, 1), origin=(0, 0, 0), chunk=1 << 22):
    """Max error of float32 points and normals against the reference's formulas
    (FlyingEdgesAlgorithm.cpp:623-647, Image3D.cpp:45-188) evaluated in
    float64 from the same float32 samples: absolute, relative to the largest
    float64 magnitude, and in float32 ulps of the float64 value."""
    nz, ny, nx = vol.shape
    axis, lo_all = edge_points(edge_of_vertex, (nx, ny, nz))
    spd, orgd = np.array(spacing, np.float64), np.array(origin, np.float64)
    res = {"points": [0.0, 0.0, 0.0], "normals": [0.0, 0.0, 0.0]}  # abs, scale, ulps

    def grad(ijk):
        g = np.zeros((len(ijk), 3))
        dims = (nx, ny, nz)
        for a in range(3):
            q0, q1 = ijk.copy(), ijk.copy()
            first = ijk[:, a] == 0
            last = ijk[:, a] == dims[a] - 1
            q0[:, a] = np.where(last, ijk[:, a], ijk[:, a] + 1)
            q1[:, a] = np.where(first, ijk[:, a], ijk[:, a] - 1)
            run = np.where(first | last, spd[a], 2 * spd[a])
            g[:, a] = (vol[q1[:, 2], q1[:, 1], q1[:, 0]].astype(np.float64) -
                       vol[q0[:, 2], q0[:, 1], q0[:, 0]].astype(np.float64)) / run
        return g

    def ulps(got, ref):
        r32 = ref.astype(np.float32)
        sp = np.abs(np.spacing(r32)).astype(np.float64)
        sp = np.where(sp > 0, sp, np.finfo(np.float32).tiny)
        return np.abs(got.astype(np.float64) - ref) / sp

    for s0 in range(0, len(axis), chunk):
        a = axis[s0:s0 + chunk]
        lo = lo_all[s0:s0 + chunk]
        d = np.stack([a == 0, a == 1, a == 2], 1).astype(np.int64)
        hi = lo + d
        v0 = vol[lo[:, 2], lo[:, 1], lo[:, 0]].astype(np.float64)
        v1 = vol[hi[:, 2], hi[:, 1], hi[:, 0]].astype(np.float64)
        w = (float(iso) - v0) / (v1 - v0)
        pos = orgd + (lo + w[:, None] * d) * spd
        g0, g1 = grad(lo), grad(hi)
        nrm = g0 + w[:, None] * (g1 - g0)
        for key, ref, got in (("points", pos, points[s0:s0 + chunk]), ("normals", nrm, normals[s0:s0 + chunk])):
            r = res[key]
            r[0] = max(r[0], float(np.abs(got - ref).max()) if len(ref) else 0.0)
            r[1] = max(r[1], float(np.abs(ref).max()) if len(ref) else 0.0)
            r[2] = max(r[2], float(ulps(got, ref).max()) if len(ref) else 0.0)
    out = {}
    for key, (err, scale, u) in res.items():
        out[key] = {"max_abs": err, "max_rel": err / scale if scale else 0.0, "max_ulps_of_fp64": u}
    return out
