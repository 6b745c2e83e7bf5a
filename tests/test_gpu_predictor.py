"""GPU: the output-size predictor's kernels against the oracle, a short
training run, and the serving loop sizing meshes with the network.

Bar: block statistics and per-block triangle counts bit-exact; the network's
output within 1e-4 and its gradient within 1e-3 of the largest component of
the float64 oracle; training beats the estimator without a network on
held-out pairs; every served mesh bit-identical to its extraction alone,
fallbacks included.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_oracle  # noqa: E402
import oracle_lib  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def dev(vol):
    import torch
    return torch.from_numpy(np.ascontiguousarray(vol, dtype=np.float32).reshape(-1)).cuda()


CASES = [((40, 33, 27), "noise", 0.0), ((17, 17, 17), "blobs", 0.5), ((16, 50, 20), "noise", 0.1),
         ((100, 37, 45), "blobs", 0.3), ((2, 2, 2), "random", 0.0), ((130, 3, 70), "random", 0.2)]


def volume(M, dims, kind, seed):
    if kind == "noise":
        return M.generate_value_noise(dims, 3, 16, seed=seed)
    if kind == "blobs":
        return M.generate_blobs(dims, 8, seed=seed)
    return np.random.default_rng(seed).standard_normal(dims[::-1]).astype(np.float32)


def test_block_stats_and_tris_match_oracle(M):
    from miniisosurface_gb300 import predictor as P
    for i, (dims, kind, iso) in enumerate(CASES):
        vol = volume(M, dims, kind, i)
        dv = dev(vol)
        st = P.block_stats(dv, dims).cpu().numpy()
        want = mlp_oracle.block_stats(vol)
        assert st.shape == want.shape
        assert np.array_equal(st.view(np.uint32), want.view(np.uint32)), dims
        tris = P.block_tris(dv, dims, iso).cpu().numpy()
        assert np.array_equal(tris, oracle_lib.block_tris(vol, iso)), dims
        assert int(tris.sum()) == M.count_device(dv, dims, iso)[1]


def test_forward_and_gradient_match_oracle(M):
    import torch
    from miniisosurface_gb300 import predictor as P
    vol = volume(M, (100, 37, 45), "noise", 9)
    st = P.block_stats(dev(vol), (100, 37, 45))
    rng = np.random.default_rng(1)
    n = st.shape[0]
    isos = torch.from_numpy(rng.uniform(-0.2, 0.2, n).astype(np.float32)).cuda()
    target = torch.from_numpy(rng.uniform(0, 5, n).astype(np.float32)).cuda()
    p = (P.init_params(3) + rng.normal(0, 0.05, P.N_PARAMS).astype(np.float32)).astype(np.float32)
    params = torch.from_numpy(p).cuda()
    x = mlp_oracle.inputs(st.cpu().numpy(), isos.cpu().numpy())
    y = P.mlp_forward(params, st, isos).cpu().numpy()
    y_ref, _ = mlp_oracle.forward(p, x)
    assert np.allclose(y, y_ref, rtol=1e-4, atol=1e-4)
    g, loss = P.mlp_gradient(params, st, isos, target)
    loss_ref, g_ref = mlp_oracle.loss_and_gradient(p, x, target.cpu().numpy())
    g = g.cpu().numpy()
    assert np.max(np.abs(g - g_ref)) <= 1e-3 * np.max(np.abs(g_ref)) + 1e-6
    assert abs(float(loss) - loss_ref) <= 1e-4 * loss_ref + 1e-6


@pytest.fixture(scope="module")
def trained(M):
    import torch
    from miniisosurface_gb300 import predictor as P
    d = torch.device("cuda", 0)
    xs, xi, xt, train_pairs = P.dataset(24, 8, seed=11, device=d)
    params = P.train(xs, xi, xt, epochs=25, batch=4096, lr=3e-3)
    pred = P.fit_margins(P.Predictor(params), train_pairs)
    return P, pred, (xs, xi, xt)


def test_training_learns_and_beats_the_estimator_without_network(M, trained):
    import torch
    P, pred, (xs, xi, xt) = trained
    init = torch.from_numpy(P.init_params(0)).cuda()
    init[-1] = float(xt.mean())
    _, loss0 = P.mlp_gradient(init, xs, xi, xt)
    _, loss1 = P.mlp_gradient(pred.params, xs, xi, xt)
    assert float(loss1) < 0.3 * float(loss0)
    _, _, _, held = P.dataset(8, 8, seed=12, device=torch.device("cuda", 0))
    ev = P.evaluate(pred, held)
    mean_per_block = float(xt.mean()) * P.LABEL_SCALE
    base = [float(((p["stats"][:, 0] < p["iso"]) & (p["stats"][:, 1] >= p["iso"])).sum()) * mean_per_block
            for p in held]
    base_err = np.median([abs(b - p["T"]) / max(p["T"], 1) for b, p in zip(base, held)])
    assert ev["rel_count_error_median"] < base_err
    assert ev["fallback_rate"] <= 0.5


def test_served_with_predictor_equals_alone(M, trained):
    from miniisosurface_gb300 import serve
    P, pred, _ = trained
    specs = [((70, 45, 50), "noise"), ((33, 90, 41), "blobs"), ((128, 40, 30), "noise")]
    vols = []
    for i, (dims, kind) in enumerate(specs):
        v = volume(M, dims, kind, 20 + i)
        lo, hi = np.percentile(v, [5, 95])
        vols.append((dev(v), dims, float(lo), float(hi)))
    volumes = [(v, d) for v, d, _, _ in vols]
    rng = np.random.default_rng(3)
    reqs = []
    for t in serve.poisson_arrivals(30, 3000.0, seed=3):
        vi = int(rng.integers(len(vols)))
        reqs.append((float(t), vi, float(np.float32(rng.uniform(vols[vi][2], vols[vi][3]))), M.FLYING_EDGES))
    # a network sized well under the truth: every request falls back to its exact sizes
    small = P.Predictor(pred.params, margin_t=0.3, v_per_t=0.3, slack=0)
    for p in (pred, small):
        server = serve.Server(volumes, slots=2, max_batch=6, lanes=2, predictor=p)
        server.inline_idle = server.single_direct = False  # every request through the network-sized batches
        server.packed = False
        server.overlap_backlog = 1
        res = server.run(reqs, keep_meshes=True)
        if p is small:
            assert server.last_fallbacks > 0
        for i, (t, vi, iso, algo) in enumerate(reqs):
            alone = M.extract_device(volumes[vi][0], volumes[vi][1], iso, algo)
            r = res[i]
            assert (r.n_points, r.n_tris) == (alone.n_points, alone.n_tris)
            assert bool((r.mesh.points[: r.n_points] == alone.points[: alone.n_points]).all())
            assert bool((r.mesh.normals[: r.n_points] == alone.normals[: alone.n_points]).all())
            assert bool((r.mesh.tris[: r.n_tris] == alone.tris[: alone.n_tris]).all())


def test_fused_prediction_matches_per_block_forward(M, trained):
    """iso_mlp_predict over several (statistics, isovalue) sets in one launch equals the
    per-block network summed over each set's active blocks."""
    import torch
    P, pred, _ = trained
    items = []
    for i, (dims, kind, _) in enumerate(CASES[:4]):
        st = P.block_stats(dev(volume(M, dims, kind, 40 + i)), dims)
        for iso in (0.0, 0.2, 0.45):
            items.append((st, iso))
    got = pred.predict(items)
    for (st, iso), g in zip(items, got):
        act = (st[:, 0] < iso) & (st[:, 1] >= iso)
        y = P.mlp_forward(pred.params, st[act].contiguous(),
                          torch.full((int(act.sum()),), iso, dtype=torch.float32, device=st.device))
        want = float(torch.clamp(y, min=0).sum()) * P.LABEL_SCALE
        assert abs(g - want) <= 1e-4 * max(want, 1.0), (g, want)


def test_extract_batch_sized_by_the_network(M, trained):
    """extract_batch with a predictor: meshes sized by the network, the batch run once (fallbacks at their exact
    sizes), every mesh equal to its plain extraction."""
    P, pred, _ = trained
    reqs = []
    for i, (dims, kind, iso) in enumerate(CASES[:4]):
        v = dev(volume(M, dims, kind, 60 + i))
        for d_iso in (0.0, 0.05):
            reqs.append(M.Request(v, dims, iso + d_iso, M.FLYING_EDGES if i % 2 == 0 else M.MARCHING_CUBES))
    for p in (pred, P.Predictor(pred.params, margin_t=0.3, v_per_t=0.3, slack=0)):  # the second always falls back
        got = M.extract_batch(reqs, predictor=p)
        for r, m in zip(reqs, got):
            alone = M.extract_device(r.volume, r.dims, r.isoval, r.algorithm)
            assert (m.n_points, m.n_tris) == (alone.n_points, alone.n_tris)
            assert bool((m.points[: m.n_points] == alone.points[: alone.n_points]).all())
            assert bool((m.tris[: m.n_tris] == alone.tris[: alone.n_tris]).all())
