"""GPU: the single-pass Flying Edges kernel (k_fe_single: counts, a single-pass
scan of the row starts, triangles and vertex records in one launch) against
the separate count / scan / generate kernels and the oracle, bit for bit.

The shapes cover the three row layouts (8, 4 and 2 rows per warp for rows
of up to 4, 8 and 16 words), row counts that do not fill the last row group,
two-point axes and tall grids; the tests also cover 64-bit indices, a mesh
that is too small (partial write, exact sizes reported), graph replay and a
grid without surface.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu

SHAPES = [
    ((40, 33, 27), "blobs", 0.5),
    ((128, 130, 31), "noise", 0.0),
    ((200, 77, 50), "noise", 0.1),
    ((256, 100, 64), "blobs", 0.4),
    ((300, 61, 40), "noise", -0.05),
    ((512, 45, 33), "noise", 0.0),
    ((4, 5, 6), "noise", 0.0),
    ((8, 2, 2), "noise", 0.0),
    ((12, 3, 200), "noise", 0.0),
    ((96, 96, 2), "blobs", 0.3),
]


def volume(M, dims, kind, seed=3):
    if kind == "blobs":
        return M.generate_blobs(dims, 8, seed=seed)
    return M.generate_value_noise(dims, 4, 16, seed=seed)


def run(M, dvol, dims, iso, single, index_bytes=4, ctx=None):
    import torch
    from miniisosurface_gb300 import _lib

    ctx = ctx or M.default_context(0)
    _lib.check(_lib.load().iso_ctx_set_single_pass(ctx.handle, 1 if single else 0), ctx.handle)
    try:
        m = M.extract_device(dvol, dims, iso, M.FLYING_EDGES, index_bytes=index_bytes, ctx=ctx)
        torch.cuda.synchronize()
        return (m.points[: m.n_points].cpu().numpy(), m.normals[: m.n_points].cpu().numpy(),
                m.tris[: m.n_tris].cpu().numpy().astype(np.uint64))
    finally:
        _lib.load().iso_ctx_set_single_pass(ctx.handle, 1)


def same(a, b, what):
    assert a[0].shape == b[0].shape and a[2].shape == b[2].shape, what
    assert np.array_equal(a[2], b[2]), what
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)), what
    assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), what


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


@pytest.mark.parametrize("dims,kind,iso", SHAPES)
def test_single_pass_equals_separate_passes(M, dims, kind, iso):
    import torch
    vol = volume(M, dims, kind)
    dv = torch.from_numpy(vol.reshape(-1)).cuda()
    one = run(M, dv, dims, iso, True)
    sep = run(M, dv, dims, iso, False)
    same(one, sep, "%s single vs separate" % (dims,))
    if np.prod(dims) <= 300_000:
        same(one, oracle_lib.fe(vol, iso)[:3], "%s single vs oracle" % (dims,))


def test_single_pass_64bit_indices_and_oracle(M):
    import torch
    dims = (200, 77, 50)
    vol = volume(M, dims, "noise", seed=9)
    dv = torch.from_numpy(vol.reshape(-1)).cuda()
    same(run(M, dv, dims, 0.0, True, index_bytes=8), oracle_lib.fe(vol, 0.0)[:3], "64-bit indices")


def test_single_pass_capacity(M):
    """A mesh one vertex or one triangle short: ISO_ERR_CAPACITY with the exact
    sizes; nothing is written past the capacities; the exact mesh then matches."""
    import torch
    from miniisosurface_gb300 import _lib

    dims = (128, 96, 64)
    vol = volume(M, dims, "blobs", seed=4)
    dv = torch.from_numpy(vol.reshape(-1)).cuda()
    ctx = M.default_context(0)
    V, T = M.count_device(dv, dims, 0.5, ctx=ctx)
    lib = _lib.load()
    g = M.make_grid(dims)
    for cv, ct in ((V - 1, T), (V, T - 1), (10, 10)):
        guard = 64
        pts = torch.full((cv + guard, 3), 7.0, device="cuda")
        nrm = torch.full((cv + guard, 3), 7.0, device="cuda")
        tri = torch.full((ct + guard, 3), 12345, dtype=torch.int32, device="cuda")
        m = _lib.IsoMesh()
        m.points, m.normals, m.tris = pts.data_ptr(), nrm.data_ptr(), tri.data_ptr()
        m.index_bytes, m.cap_points, m.cap_tris = 4, cv, ct
        st = lib.iso_extract_device(ctx.handle, M.FLYING_EDGES, dv.data_ptr(), C.byref(g), C.c_float(0.5),
                                    C.byref(m), None)
        torch.cuda.synchronize()
        assert st == _lib.ISO_ERR_CAPACITY
        assert (m.n_points, m.n_tris) == (V, T)
        assert bool((pts[cv:] == 7.0).all()) and bool((nrm[cv:] == 7.0).all())
        assert bool((tri[ct:] == 12345).all())
    same(run(M, dv, dims, 0.5, True), oracle_lib.fe(vol, 0.5)[:3], "after capacity errors")


def test_single_pass_graph_replay(M):
    import torch
    from miniisosurface_gb300 import _lib

    dims = (256, 100, 64)
    vol = volume(M, dims, "noise", seed=5)
    dv = torch.from_numpy(vol.reshape(-1)).cuda()
    ctx = M.Context(0)
    lib = _lib.load()
    V, T = M.count_device(dv, dims, 0.0, ctx=ctx)
    out = M.DeviceMesh(V, T, 4)
    desc = out.descriptor()
    res = torch.zeros(4, dtype=torch.int64).pin_memory()
    g = M.make_grid(dims)
    lib.iso_ctx_set_graph(ctx.handle, 1)
    ref = oracle_lib.fe(vol, 0.0)[:3]
    for rep in range(3):
        out.points.fill_(0.0)
        out.tris.fill_(-1)
        st = lib.iso_extract_device_async(ctx.handle, M.FLYING_EDGES, dv.data_ptr(), C.byref(g), C.c_float(0.0),
                                          C.byref(desc), C.c_void_p(res.data_ptr()), None)
        assert st == 0
        torch.cuda.synchronize()
        assert (int(res[0]), int(res[1]), int(res[3])) == (V, T, 0)
        same((out.points[:V].cpu().numpy(), out.normals[:V].cpu().numpy(),
              out.tris[:T].cpu().numpy().astype(np.uint64)), ref, "graph replay %d" % rep)
    lib.iso_ctx_set_graph(ctx.handle, 0)


def test_single_pass_no_surface(M):
    import torch
    dims = (64, 40, 30)
    dv = torch.full((64 * 40 * 30,), 2.0, device="cuda")
    p, n, t = run(M, dv, dims, 0.5, True)
    assert p.shape == (0, 3) and t.shape == (0, 3)
