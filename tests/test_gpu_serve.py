"""GPU: the serving loop (continuous batching over two slots) against each
request extracted alone, and against the plain one-at-a-time loop.

Bar: every request's mesh bit-identical alone, in the plain loop and in the
mix of batches, whatever batch and slot it landed in.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def as_np(m):
    return (m.points[: m.n_points].cpu().numpy().view(np.uint32), m.normals[: m.n_points].cpu().numpy().view(np.uint32),
            m.tris[: m.n_tris].cpu().numpy().astype(np.uint64))


def pool(M):
    import torch
    specs = [((70, 45, 50), "noise"), ((33, 90, 41), "blobs"), ((128, 40, 30), "noise"), ((57, 57, 57), "blobs")]
    vols = []
    for i, (dims, kind) in enumerate(specs):
        v = M.generate_value_noise(dims, 3, 16, seed=i) if kind == "noise" else M.generate_blobs(dims, 8, seed=i)
        lo, hi = np.percentile(v, [5, 95])
        vols.append((torch.from_numpy(v.reshape(-1)).cuda(), dims, float(lo), float(hi)))
    return vols


def test_served_equals_alone_and_plain(M):
    from miniisosurface_gb300 import serve
    vols = pool(M)
    volumes = [(v, d) for v, d, _, _ in vols]
    rng = np.random.default_rng(5)
    arrivals = serve.poisson_arrivals(48, 4000.0, seed=5)
    reqs = []
    for t in arrivals:
        vi = int(rng.integers(len(vols)))
        lo, hi = vols[vi][2], vols[vi][3]
        algo = M.FLYING_EDGES if rng.random() < 0.75 else M.MARCHING_CUBES
        reqs.append((float(t), vi, float(np.float32(rng.uniform(lo, hi))), algo))
    # a budget of about three average meshes: admission holds requests back while others run
    sizes = [M.count_device(volumes[vi][0], volumes[vi][1], iso, algo) for _, vi, iso, algo in reqs]
    budget = 3 * int(np.mean([serve.mesh_bytes(v, t) for v, t in sizes]))
    server = serve.Server(volumes, slots=2, max_batch=8, budget_bytes=budget, lanes=3)
    # continuous batching itself: every request through the slots' batches, a slot starting beside a running
    # one as soon as anything waits
    server.inline_idle = server.single_direct = False
    server.overlap_backlog = 1
    served = server.run(reqs, keep_meshes=True)
    server.inline_idle = server.single_direct = True
    server.overlap_backlog = 4
    plain = serve.run_plain(volumes, reqs, keep_meshes=True)
    assert max(np.bincount([r.batch for r in served])) > 1, "no batch held more than one request"
    # light load (the defaults): requests that find the server idle run at once on the receiving thread, a
    # slot starts beside running work only behind a backlog; the same meshes
    slow = [(float(t) * 40.0, vi, iso, algo) for t, vi, iso, algo in reqs[:6]]
    light = server.run(slow, keep_meshes=True)
    assert any(r.slot == -1 for r in light), "no request ran on the receiving thread"
    for i, (t, vi, iso, algo) in enumerate(slow):
        ref = M.extract_device(volumes[vi][0], volumes[vi][1], iso, algo)
        assert (light[i].n_points, light[i].n_tris) == (ref.n_points, ref.n_tris)
        for x, y in zip(as_np(light[i].mesh), as_np(ref)):
            assert np.array_equal(x, y), "light-load request %d differs" % i
    assert len({r.slot for r in served if r.slot >= 0}) == 2, "one slot did all the work"
    for i, (t, vi, iso, algo) in enumerate(reqs):
        alone = M.extract_device(volumes[vi][0], volumes[vi][1], iso, algo)
        a = as_np(alone)
        for name, r in (("served", served[i]), ("plain", plain[i])):
            assert (r.n_points, r.n_tris) == sizes[i]
            for x, y in zip(as_np(r.mesh), a):
                assert np.array_equal(x, y), "%s request %d differs from its extraction alone" % (name, i)
        assert served[i].latency > 0 and plain[i].latency > 0
    cells = [int(np.prod([d - 1 for d in volumes[vi][1]])) for _, vi, _, _ in reqs]
    s = serve.summary(served, cells)
    assert s["p99_ms"] >= s["p50_ms"] > 0


def test_concurrent_contexts_agree(M):
    """Two contexts on two host threads extract batches at once, meshes freed every round: the widths 70 and 57
    run the same count kernel with different shared-memory sizes, so one thread's launch setting must never
    affect the other's.  Every request's status and counts must equal count_device."""
    import threading
    import torch
    vols = pool(M)
    volumes = [(v, d) for v, d, _, _ in vols]
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(24):
        vi = (0, 3)[i % 2]  # 70 and 57 points wide
        algo = M.FLYING_EDGES if i % 4 < 3 else M.MARCHING_CUBES
        reqs.append((vi, float(np.float32(rng.uniform(vols[vi][2], vols[vi][3]))), algo))
    ref = [M.count_device(volumes[vi][0], volumes[vi][1], iso, algo) for vi, iso, algo in reqs]
    bad, errors = [], []

    def work(seed):
        try:
            ctx = M.Context(0)
            M.set_batch_lanes(3, ctx)
            M.set_batch_graph(False, ctx)
            s = torch.cuda.Stream()
            r = np.random.default_rng(seed)
            for it in range(80):
                pick = r.choice(len(reqs), int(r.integers(1, 7)), replace=False)
                rs = [M.Request(volumes[reqs[i][0]][0], volumes[reqs[i][0]][1], reqs[i][1], reqs[i][2]) for i in pick]
                with torch.cuda.stream(s):
                    ms = [M.DeviceMesh(ref[i][0], ref[i][1], 4) for i in pick]
                codes = M.Batch(rs, ms).run(ctx, s.cuda_stream)
                for q, i in enumerate(pick):
                    if codes[q] != 0 or (ms[q].n_points, ms[q].n_tris) != ref[i]:
                        bad.append((seed, it, int(i), ref[i], (ms[q].n_points, ms[q].n_tris), codes[q]))
        except Exception as e:  # noqa: BLE001 -- reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(k,)) for k in (1, 2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:2]
    assert not bad, bad[:4]
