"""GPU: batched extraction (iso_extract_batch) against one iso_extract_device
call per request and against the oracle.

Bar: every request's mesh bit-identical to its own plain extraction (points,
normals, connectivity, counts), whatever the lanes, and the same after the
captured graph is replayed or updated.
"""
import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu


def dev(vol):
    import torch
    return torch.from_numpy(np.ascontiguousarray(vol, dtype=np.float32).reshape(-1)).cuda()


def as_np(m):
    return (m.points[: m.n_points].cpu().numpy(), m.normals[: m.n_points].cpu().numpy(),
            m.tris[: m.n_tris].cpu().numpy().astype(np.uint64))


def same(a, b, what):
    for x, y, name in zip(a, b, ("points", "normals", "triangles")):
        assert x.shape == y.shape, "%s: %s shape %s vs %s" % (what, name, x.shape, y.shape)
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y), "%s: %s differ" % (what, name)


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def mixed_requests(M):
    """Requests over every kernel choice: 1-4, 5-8 and 9-16 word rows, rows of
    17-32 words (one row per warp) and longer (row kernels), unaligned widths,
    two-point grids, an empty grid and a volume without surface."""
    rng = np.random.default_rng(7)
    specs = [
        ((40, 33, 27), "blobs", 0.5, M.FLYING_EDGES, 4, (0.1, 0.37, 1.3), (-2.5, 0.3, 7.1)),
        ((61, 47, 35), "noise", 0.0, M.MARCHING_CUBES, 4, (1, 1, 1), (0, 0, 0)),
        ((64, 20, 20), "noise", 0.05, M.MC_DUPFREE, 8, (1, 1, 1), (0, 0, 0)),
        ((600, 9, 7), "noise", 0.0, M.FLYING_EDGES, 8, (1, 1, 1), (0, 0, 0)),
        ((1029, 3, 3), "noise", 0.1, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
        ((127, 30, 20), "noise", 0.0, M.MARCHING_CUBES, 8, (0.5, 1.5, 0.75), (1.0, -2.0, 0.5)),
        ((2, 2, 2), "random", 0.0, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
        ((1, 5, 5), "random", 0.0, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
        ((33, 2, 2), "random", 0.1, M.MARCHING_CUBES, 4, (1, 1, 1), (0, 0, 0)),
        ((128, 64, 40), "blobs", 0.5, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
        ((45, 33, 28), "noise", 5.0, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
        ((256, 31, 17), "noise", -0.1, M.FLYING_EDGES, 4, (1, 1, 1), (0, 0, 0)),
    ]
    reqs, vols = [], []
    for i, (dims, field, iso, algo, ib, sp, org) in enumerate(specs):
        nx, ny, nz = dims
        if field == "blobs":
            vol = M.generate_blobs(dims, 8, seed=i)
        elif field == "noise":
            vol = M.generate_value_noise(dims, 3, 16, seed=i)
        else:
            vol = rng.standard_normal((nz, ny, nx)).astype(np.float32)
        vols.append(vol)
        reqs.append((M.Request(dev(vol), dims, iso, algo, sp, org), ib))
    return reqs, vols


def plain(M, r, ib):
    return as_np(M.extract_device(r.volume, r.dims, r.isoval, r.algorithm, r.spacing, r.origin, index_bytes=ib))


def test_batch_matches_plain_and_oracle(M):
    reqs, vols = mixed_requests(M)
    M.set_batch_lanes(3)
    meshes = [M.DeviceMesh(0, 0, ib) for _, ib in reqs]
    got = M.extract_batch([r for r, _ in reqs], meshes)
    for i, ((r, ib), m) in enumerate(zip(reqs, got)):
        same(as_np(m), plain(M, r, ib), "request %d %s" % (i, r.dims))
    # three against the oracle directly
    for i in (0, 1, 5):
        r = reqs[i][0]
        ref = (oracle_lib.fe if r.algorithm == M.FLYING_EDGES else oracle_lib.mc)(vols[i], r.isoval, r.spacing,
                                                                                    r.origin)
        p, n, t = as_np(got[i])
        assert np.array_equal(t, ref[2].astype(np.uint64))
        assert np.array_equal(p.view(np.uint32), ref[0].view(np.uint32))
        assert np.array_equal(n.view(np.uint32), ref[1].view(np.uint32))


def test_lanes_and_autotuner_agree(M):
    reqs, _ = mixed_requests(M)
    want = None
    for lanes, graph, share in ((1, True, 1), (4, True, 4), (0, True, 0), (3, False, 2), (1, False, 1),
                                (5, True, 8)):
        M.set_batch_lanes(lanes)
        M.set_batch_split(share)
        M.set_batch_graph(graph)
        got = [as_np(m) for m in M.extract_batch([r for r, _ in reqs], [M.DeviceMesh(0, 0, ib) for _, ib in reqs])]
        if lanes == 0:
            assert M.batch_lanes() in (1, 2, 4, 8, 16, 32, 64)
            assert M.batch_split() in (1, 2, 4, 8) and M.batch_split() <= M.batch_lanes()
        if want is None:
            want = got
        else:
            for i, (a, b) in enumerate(zip(got, want)):
                same(a, b, "lanes %d graph %s split %d request %d" % (lanes, graph, share, i))
    M.set_batch_graph(True)
    M.set_batch_lanes(0)
    M.set_batch_split(0)


def test_capacity_per_request(M):
    from miniisosurface_gb300 import _lib
    reqs, _ = mixed_requests(M)
    rs = [r for r, _ in reqs]
    sizes = [M.count_device(r.volume, r.dims, r.isoval, r.algorithm) for r in rs]
    meshes = [M.DeviceMesh(v, t, ib) for (v, t), (_, ib) in zip(sizes, reqs)]
    small = 1  # too few points for request 1
    meshes[small] = M.DeviceMesh(sizes[small][0] - 1, sizes[small][1], reqs[small][1])
    codes = M.Batch(rs, meshes).run()
    for i, c in enumerate(codes):
        assert c == (_lib.ISO_ERR_CAPACITY if i == small else _lib.ISO_OK), (i, c)
        assert (meshes[i].n_points, meshes[i].n_tris) == sizes[i]
        if i != small:
            same(as_np(meshes[i]), plain(M, rs[i], reqs[i][1]), "request %d" % i)


def test_replay_and_update(M):
    reqs, _ = mixed_requests(M)
    rs = [r for r, _ in reqs]
    M.set_batch_lanes(2)
    meshes = M.extract_batch(rs, [M.DeviceMesh(0, 0, ib) for _, ib in reqs])
    b = M.Batch(rs, meshes)
    first = [as_np(m) for m in meshes]
    for m in meshes:  # poison the outputs: the replayed graph must rewrite them
        m.points.fill_(7.0)
        m.tris.fill_(-1)
    assert all(c == 0 for c in b.run())
    for i, (m, f) in enumerate(zip(meshes, first)):
        same(as_np(m), f, "replay %d" % i)
    # a changed isovalue: the graph is captured again and updated in place
    rs2 = list(rs)
    r0 = rs[0]
    rs2[0] = M.Request(r0.volume, r0.dims, 0.45, r0.algorithm, r0.spacing, r0.origin)
    meshes2 = M.extract_batch(rs2, [M.DeviceMesh(0, 0, ib) for _, ib in reqs])
    same(as_np(meshes2[0]), plain(M, rs2[0], reqs[0][1]), "updated request 0")
    for i in range(1, len(rs)):
        same(as_np(meshes2[i]), first[i], "updated batch request %d" % i)
    M.set_batch_lanes(0)


def test_one_shot_graph_mode(M):
    """iso_ctx_set_graph: repeated device extractions relaunch a captured graph; a changed isovalue, mesh or
    algorithm captures again; every mesh equals the stream path's."""
    import torch
    reqs, _ = mixed_requests(M)
    ctx = M.Context(0)
    picks = [reqs[i] for i in (0, 1, 3, 9, 11)]
    want = [plain(M, r, ib) for r, ib in picks]
    M.set_graph(True, ctx)
    try:
        for rep in range(3):
            for (r, ib), w in zip(picks, want):
                m = M.DeviceMesh(len(w[0]), len(w[2]), ib)
                for _ in range(2):  # the second call relaunches the graph of the first
                    m.points.fill_(3.0)
                    got = M.extract_device(r.volume, r.dims, r.isoval, r.algorithm, r.spacing, r.origin, out=m,
                                           index_bytes=ib, ctx=ctx)
                    torch.cuda.synchronize()
                    same(as_np(got), w, "graph mode %s rep %d" % (r.dims, rep))
    finally:
        M.set_graph(False, ctx)


def test_batch_edge_cases(M):
    """Empty batches, an invalid request beside valid ones (only it fails), a mesh with a bad index width, and
    the count-only batch against count_device."""
    import ctypes as C
    from miniisosurface_gb300 import _lib
    lib = _lib.load()
    ctx = M.Context(0)
    assert M.extract_batch([], ctx=ctx) == []
    assert lib.iso_extract_batch(ctx.handle, 0, None, None, None, None) == _lib.ISO_OK
    assert lib.iso_extract_batch(ctx.handle, -1, None, None, None, None) == _lib.ISO_ERR_INVALID_ARG
    assert lib.iso_count_batch(ctx.handle, 2, None, None, None, None, None) == _lib.ISO_ERR_INVALID_ARG
    reqs, _ = mixed_requests(M)
    rs = [r for r, _ in reqs][:4]
    sizes = [M.count_device(r.volume, r.dims, r.isoval, r.algorithm) for r in rs]
    meshes = [M.DeviceMesh(v, t, 4) for v, t in sizes]
    b = M.Batch(rs, meshes)
    b.req[1].algorithm = 7  # no such algorithm
    b.out[2].index_bytes = 3  # no such index width
    st = lib.iso_extract_batch(ctx.handle, len(rs), b.req, b.out, b.status, None)
    codes = [b.status[i] for i in range(len(rs))]
    assert st == _lib.ISO_ERR_INVALID_ARG
    assert codes == [_lib.ISO_OK, _lib.ISO_ERR_INVALID_ARG, _lib.ISO_ERR_INVALID_ARG, _lib.ISO_OK]
    for i in (0, 3):
        assert (b.out[i].n_points, b.out[i].n_tris) == sizes[i]
        meshes[i].n_points, meshes[i].n_tris = b.out[i].n_points, b.out[i].n_tris
        same(as_np(meshes[i]), plain(M, rs[i], 4), "edge-case batch request %d" % i)
    allr = [r for r, _ in reqs]
    arr = (_lib.IsoRequest * len(allr))(*[r.descriptor() for r in allr])
    nv, nt = (C.c_int64 * len(allr))(), (C.c_int64 * len(allr))()
    assert lib.iso_count_batch(ctx.handle, len(allr), arr, nv, nt, None, None) == _lib.ISO_OK
    for i, r in enumerate(allr):
        assert (nv[i], nt[i]) == M.count_device(r.volume, r.dims, r.isoval, r.algorithm), r.dims
