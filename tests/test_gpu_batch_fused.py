"""GPU: fused batches (iso_batch_set_fused, batch_kernels.cuh) -- the Flying
Edges requests of rows up to 512 points run one launch per pass -- against the
same batch on the lanes, against one iso_extract_device call per request and
against the oracle.

Bar: every request's mesh and counts bit-identical, whatever the count
variant (rows per warp 8 / 4 / 2, row length a multiple of 4 points or not,
rows of exactly 128 / 256 / 512 points), index width, graph or direct launch,
with requests on the lanes beside them (Marching Cubes, long rows, a volume
not at a 16-byte boundary), a mesh too small for its counts, and more than
1,024 requests (several per thread of the vertex prefix).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu

WIDTHS = [37, 64, 128, 150, 160, 256, 301, 300, 512]  # every count variant of rows up to 16 words


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def dev(vol):
    import torch
    return torch.from_numpy(np.ascontiguousarray(vol, dtype=np.float32).reshape(-1)).cuda()


def as_np(m):
    return (m.points[: m.n_points].cpu().numpy().view(np.uint32), m.normals[: m.n_points].cpu().numpy().view(np.uint32),
            m.tris[: m.n_tris].cpu().numpy().astype(np.uint64))


def same(a, b, what):
    for x, y, name in zip(a, b, ("points", "normals", "triangles")):
        assert x.shape == y.shape, "%s: %s shape %s vs %s" % (what, name, x.shape, y.shape)
        assert np.array_equal(x, y), "%s: %s differ" % (what, name)


def requests(M):
    """(request, index bytes, host volume): the nine widths, two index widths, blobs and noise, spacing and
    origin, with lane requests mixed in."""
    import torch
    out = []
    for i, nx in enumerate(WIDTHS):
        dims = (nx, 20 + 7 * i, 11 + 3 * i)
        vol = M.generate_blobs(dims, 6, seed=i) if i % 2 else M.generate_value_noise(dims, 3, 16, seed=i)
        lo, hi = np.percentile(vol, [20, 80])
        iso = float(np.float32(lo + (hi - lo) * (0.3 + 0.05 * i)))
        sp = (1.0, 1.0, 1.0) if i % 3 else (0.5, 1.25, 2.0)
        org = (0.0, 0.0, 0.0) if i % 4 else (-3.0, 1.5, 0.25)
        out.append((M.Request(dev(vol), dims, iso, M.FLYING_EDGES, sp, org), 8 if i % 4 == 3 else 4, vol))
    # on the lanes: Marching Cubes, rows longer than 16 words, a volume one sample past a 16-byte boundary
    v = M.generate_value_noise((70, 30, 25), 3, 16, seed=40)
    out.append((M.Request(dev(v), (70, 30, 25), 0.0, M.MARCHING_CUBES), 4, v))
    v = M.generate_value_noise((700, 12, 9), 3, 16, seed=41)
    out.append((M.Request(dev(v), (700, 12, 9), 0.0, M.FLYING_EDGES), 4, v))
    v = M.generate_value_noise((96, 40, 30), 3, 16, seed=42)
    flat = torch.zeros(v.size + 1, dtype=torch.float32, device="cuda")
    flat[1:] = dev(v)
    out.append((M.Request(flat[1:], (96, 40, 30), 0.0, M.FLYING_EDGES), 4, v))
    # no surface, and a two-point grid
    v = M.generate_value_noise((48, 20, 10), 3, 16, seed=43)
    out.append((M.Request(dev(v), (48, 20, 10), 10.0, M.FLYING_EDGES), 4, v))
    v = np.array([[[0.0, 1.0], [1.0, 0.0]], [[1.0, 0.0], [0.0, 1.0]]], dtype=np.float32)
    out.append((M.Request(dev(v), (2, 2, 2), 0.5, M.FLYING_EDGES), 4, v))
    return out


def run(M, reqs, mode, graph=True, lanes=3, ctx=None):
    """The batch with iso_batch_set_fused(mode): 0 lanes, 1 the default, 2 always fused."""
    ctx = ctx or M.default_context()
    M.set_batch_fused(mode, ctx)
    M.set_batch_graph(graph, ctx)
    M.set_batch_lanes(lanes, ctx)
    M.set_batch_split(1, ctx)
    try:
        return [as_np(m) for m in M.extract_batch([r for r, _, _ in reqs], [M.DeviceMesh(0, 0, ib) for _, ib, _ in reqs],
                                                  ctx=ctx)]
    finally:
        M.set_batch_fused(True, ctx)
        M.set_batch_graph(True, ctx)
        M.set_batch_lanes(0, ctx)
        M.set_batch_split(0, ctx)


def test_fused_equals_lanes_plain_and_oracle(M):
    reqs = requests(M)
    fused = run(M, reqs, 2)
    lanes = run(M, reqs, 0)
    direct = run(M, reqs, 2, graph=False)
    auto = run(M, reqs, 1)  # the default: 9 requests qualify, fewer than 16, so all of them on the lanes
    for i, ((r, ib, vol), a, b, c, d) in enumerate(zip(reqs, fused, lanes, direct, auto)):
        what = "request %d %s" % (i, r.dims)
        same(a, b, what + " fused vs lanes")
        same(a, d, what + " fused vs default")
        same(a, c, what + " graph vs direct")
        p = M.extract_device(r.volume, r.dims, r.isoval, r.algorithm, r.spacing, r.origin, index_bytes=ib)
        same(a, as_np(p), what + " fused vs plain")
    for i in (0, 4, 8):  # unaligned 8 rows per warp, aligned 4, full 2
        r, ib, vol = reqs[i]
        ref = oracle_lib.fe(vol, r.isoval, r.spacing, r.origin)
        same(fused[i], (ref[0].view(np.uint32), ref[1].view(np.uint32), ref[2].astype(np.uint64)),
             "request %d vs oracle" % i)


def test_fused_capacity_replay_and_counts(M):
    from miniisosurface_gb300 import _lib
    lib = _lib.load()
    reqs = requests(M)
    rs = [r for r, _, _ in reqs]
    sizes = [M.count_device(r.volume, r.dims, r.isoval, r.algorithm) for r in rs]
    ctx = M.Context(0)
    M.set_batch_lanes(2, ctx)
    M.set_batch_split(1, ctx)
    M.set_batch_fused(2, ctx)
    meshes = [M.DeviceMesh(v, t, ib) for (v, t), (_, ib, _) in zip(sizes, reqs)]
    small, small_t = 2, 5  # fused requests: one point too few, one triangle too few
    meshes[small] = M.DeviceMesh(sizes[small][0] - 1, sizes[small][1], reqs[small][1])
    meshes[small_t] = M.DeviceMesh(sizes[small_t][0], sizes[small_t][1] - 1, reqs[small_t][1])
    b = M.Batch(rs, meshes)
    want = [as_np(M.extract_device(r.volume, r.dims, r.isoval, r.algorithm, r.spacing, r.origin, index_bytes=ib))
            for r, ib, _ in reqs]
    for rep in range(3):  # capture, then replays of the graph over poisoned outputs
        for m in meshes:
            if m.points.numel():
                m.points.fill_(7.0)
            if m.tris.numel():
                m.tris.fill_(-1)
        codes = b.run(ctx)
        for i, c in enumerate(codes):
            bad = i in (small, small_t)
            assert c == (_lib.ISO_ERR_CAPACITY if bad else _lib.ISO_OK), (rep, i, c)
            assert (meshes[i].n_points, meshes[i].n_tris) == sizes[i], (rep, i)
            if not bad:
                same(as_np(meshes[i]), want[i], "rep %d request %d" % (rep, i))
    # counts only, fused and on the lanes
    arr = (_lib.IsoRequest * len(rs))(*[r.descriptor() for r in rs])
    for fused in (2, 0):
        lib.iso_batch_set_fused(ctx.handle, fused)
        nv, nt = (C.c_int64 * len(rs))(), (C.c_int64 * len(rs))()
        assert lib.iso_count_batch(ctx.handle, len(rs), arr, nv, nt, None, None) == _lib.ISO_OK
        assert [(nv[i], nt[i]) for i in range(len(rs))] == sizes, fused
    lib.iso_batch_set_fused(ctx.handle, 1)
    assert lib.iso_batch_set_fused(ctx.handle, 3) == _lib.ISO_ERR_INVALID_ARG


def test_fused_many_requests(M):
    """1,100 small requests over 25 volumes (several per thread of the vertex prefix), direct launch, fused by
    default (more than 16 requests)."""
    import torch
    rng = np.random.default_rng(3)
    vols = []
    for v in range(25):
        dims = tuple(int(x) for x in rng.integers(6, 40, size=3))
        vols.append((dims, dev(M.generate_value_noise(dims, 2, 8, seed=100 + v))))
    reqs = []
    for q in range(1100):
        dims, dv = vols[q % len(vols)]
        reqs.append((M.Request(dv, dims, float(np.float32(rng.uniform(-0.3, 0.3))), M.FLYING_EDGES), 4, None))
    fused = run(M, reqs, 1, graph=False, lanes=4)
    lanes = run(M, reqs, 0, graph=False, lanes=4)
    for i, (a, b) in enumerate(zip(fused, lanes)):
        same(a, b, "request %d" % i)
    for i in range(0, 1100, 97):
        r = reqs[i][0]
        same(fused[i], as_np(M.extract_device(r.volume, r.dims, r.isoval)), "request %d vs plain" % i)
    torch.cuda.synchronize()


def test_packed_batch(M):
    """iso_extract_batch_packed: the fused requests' meshes one after another in one set of buffers, each
    equal to its own extraction; a capacity that holds the first three meshes; requests the packed batch
    does not take; the Python helper growing its buffers."""
    from miniisosurface_gb300 import _lib
    lib = _lib.load()
    reqs = requests(M)
    take = [q for q, (r, _, _) in enumerate(reqs) if r.algorithm == M.FLYING_EDGES and r.dims[0] <= 512 and
            r.volume.data_ptr() % 16 == 0]
    rs = [reqs[q][0] for q in take]
    want = [as_np(M.extract_device(r.volume, r.dims, r.isoval, r.algorithm, r.spacing, r.origin, index_bytes=ib))
            for r, ib in ((reqs[q][0], reqs[q][1]) for q in take)]
    for ib in (4, 8):
        meshes, bufs = M.extract_batch_packed(rs, index_bytes=ib)
        at_v = at_t = 0
        for q, (m, w) in enumerate(zip(meshes, want)):
            same(as_np(m), w, "packed request %d, %d-byte indices" % (q, ib))
            assert m.points.data_ptr() == bufs.points.data_ptr() + 12 * at_v  # one after another
            assert m.tris.data_ptr() == bufs.tris.data_ptr() + 3 * ib * at_t
            at_v += m.n_points
            at_t += m.n_tris
        meshes2, bufs2 = M.extract_batch_packed(rs, buffers=bufs, index_bytes=ib)  # reused, no growth
        assert bufs2 is bufs and bufs2.points.data_ptr() == bufs.points.data_ptr()
        for q, (m, w) in enumerate(zip(meshes2, want)):
            same(as_np(m), w, "packed again request %d" % q)
    # room for the first three meshes only
    n = len(rs)
    nv = [len(w[0]) for w in want]
    nt = [len(w[2]) for w in want]
    cap_p, cap_t = sum(nv[:3]), sum(nt[:3])
    bufs = M.PackedBuffers(cap_p, cap_t, 4)
    arr = (_lib.IsoRequest * n)(*[r.descriptor() for r in rs])
    pf, tf, gv, gt = [(C.c_int64 * n)() for _ in range(4)]
    st = (C.c_int * n)()
    rc = lib.iso_extract_batch_packed(M.default_context().handle, n, arr, bufs.points.data_ptr(),
                                      bufs.normals.data_ptr(), bufs.tris.data_ptr(), 4, cap_p, cap_t, pf, tf, gv, gt,
                                      st, None)
    assert rc == _lib.ISO_ERR_CAPACITY
    for q in range(n):
        assert (gv[q], gt[q]) == (nv[q], nt[q]) and pf[q] == sum(nv[:q]) and tf[q] == sum(nt[:q])
        placed = pf[q] + nv[q] <= cap_p and tf[q] + nt[q] <= cap_t
        assert st[q] == (_lib.ISO_OK if placed else _lib.ISO_ERR_CAPACITY), q
        if placed:
            got = (bufs.points[pf[q]: pf[q] + nv[q]].cpu().numpy().view(np.uint32),
                   bufs.normals[pf[q]: pf[q] + nv[q]].cpu().numpy().view(np.uint32),
                   bufs.tris[tf[q]: tf[q] + nt[q]].cpu().numpy().astype(np.uint64))
            same(got, want[q], "capacity-limited request %d" % q)
    # the whole list: the requests outside the packed path are refused, the rest complete
    alln = len(reqs)
    arr = (_lib.IsoRequest * alln)(*[r.descriptor() for r, _, _ in reqs])
    pf, tf, gv, gt = [(C.c_int64 * alln)() for _ in range(4)]
    st = (C.c_int * alln)()
    bufs = M.PackedBuffers(sum(nv), sum(nt), 4)
    rc = lib.iso_extract_batch_packed(M.default_context().handle, alln, arr, bufs.points.data_ptr(),
                                      bufs.normals.data_ptr(), bufs.tris.data_ptr(), 4, bufs.points.shape[0],
                                      bufs.tris.shape[0], pf, tf, gv, gt, st, None)
    assert rc == _lib.ISO_ERR_INVALID_ARG
    k = 0
    for q in range(alln):
        if q in take:
            assert st[q] == _lib.ISO_OK
            got = (bufs.points[pf[q]: pf[q] + gv[q]].cpu().numpy().view(np.uint32),
                   bufs.normals[pf[q]: pf[q] + gv[q]].cpu().numpy().view(np.uint32),
                   bufs.tris[tf[q]: tf[q] + gt[q]].cpu().numpy().astype(np.uint64))
            same(got, want[k], "mixed list request %d" % q)
            k += 1
        elif reqs[q][0].dims == (2, 2, 2) or reqs[q][0].dims[0] < 2:
            pass
        else:
            assert st[q] == _lib.ISO_ERR_INVALID_ARG, q


def test_packed_many_requests(M):
    rng = np.random.default_rng(5)
    vols = []
    for v in range(20):
        dims = tuple(int(x) for x in rng.integers(6, 60, size=3))
        vols.append((dims, dev(M.generate_value_noise(dims, 2, 8, seed=300 + v))))
    rs = [M.Request(vols[q % 20][1], vols[q % 20][0], float(np.float32(rng.uniform(-0.3, 0.3)))) for q in range(1500)]
    meshes, _ = M.extract_batch_packed(rs)
    for q in range(0, 1500, 61):
        r = rs[q]
        same(as_np(meshes[q]), as_np(M.extract_device(r.volume, r.dims, r.isoval)), "request %d" % q)


def test_fused_split_autotuner(M):
    """The first graph-mode batch with fused requests times the fused work splits and keeps one of them; the
    meshes equal the plain calls' whatever split it keeps."""
    rng = np.random.default_rng(11)
    rs = []
    for q in range(20):
        dims = tuple(int(x) for x in rng.integers(20, 140, size=3))
        rs.append(M.Request(dev(M.generate_value_noise(dims, 3, 16, seed=500 + q)), dims, 0.0))
    ctx = M.Context(0)
    M.set_batch_lanes(0, ctx)
    assert M.batch_fused_split(ctx) == (0, 0)
    # meshes of the exact sizes, so that every candidate's graph runs the generate and vertex passes too (each
    # candidate has its own launch geometry: its graph must be captured anew, not replayed)
    sizes = [M.count_device(r.volume, r.dims, r.isoval, ctx=ctx) for r in rs]
    meshes = [M.DeviceMesh(v, t, 4) for v, t in sizes]
    assert all(c == 0 for c in M.Batch(rs, meshes).run(ctx))
    kc, ipw = M.batch_fused_split(ctx)
    assert kc in (8, 16, 32) and ipw in (16, 32, 64), (kc, ipw)
    for q, (r, m) in enumerate(zip(rs, meshes)):
        same(as_np(m), as_np(M.extract_device(r.volume, r.dims, r.isoval)), "request %d" % q)
    M.set_batch_lanes(0, ctx)  # tunes again on the next batch
    assert M.batch_fused_split(ctx) == (0, 0)
