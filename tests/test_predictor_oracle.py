"""CPU: the output-size predictor's oracle pinned on its own -- the numpy
gradient against finite differences, the per-block triangle counts against
the Flying Edges oracle's mesh."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_oracle  # noqa: E402
import oracle_lib  # noqa: E402


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, mlp_oracle.N_PARAMS)
    x = rng.normal(0, 1, (40, mlp_oracle.N_IN))
    t = rng.normal(0, 1, 40)
    loss, g = mlp_oracle.loss_and_gradient(p, x, t)
    idx = rng.choice(mlp_oracle.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [mlp_oracle.N_PARAMS - 1]])  # b3 too
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = mlp_oracle.loss_and_gradient(q, x, t)
        q[i] -= 2 * h
        lm, _ = mlp_oracle.loss_and_gradient(q, x, t)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_block_tris_sum_to_the_mesh():
    import miniisosurface_gb300 as M  # host generators only
    for dims, iso, seed in (((40, 33, 27), 0.0, 1), ((17, 50, 33), 0.1, 2), ((70, 16, 18), -0.05, 3)):
        vol = M.generate_value_noise(dims, 3, 16, seed=seed)
        counts = oracle_lib.block_tris(vol, iso)
        nb = [(n - 2) // 16 + 1 for n in dims]
        assert counts.size == nb[0] * nb[1] * nb[2]
        assert int(counts.sum()) == oracle_lib.fe(vol, iso)[2].shape[0]


def test_block_stats_histogram_sums_to_one():
    rng = np.random.default_rng(4)
    vol = rng.standard_normal((20, 35, 18)).astype(np.float32)
    st = mlp_oracle.block_stats(vol)
    assert st.shape == (2 * 3 * 2, 34)
    assert np.allclose(st[:, 2:].sum(1), 1.0, atol=1e-5)
    assert np.all(st[:, 0] <= st[:, 1])
