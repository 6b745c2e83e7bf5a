"""Serving loop host logic on CPU: admission by output bytes, Poisson arrivals,
meshes carved from one allocation per batch, the output-size network's
capacity rule."""
import numpy as np
import pytest

from miniisosurface_gb300.serve import admit, mesh_bytes, poisson_arrivals


def test_mesh_bytes():
    assert mesh_bytes(10, 7) == 24 * 10 + 12 * 7
    assert mesh_bytes(10, 7, 8) == 24 * 10 + 24 * 7


def test_admit_prefix_under_budget():
    sizes = [(100, 200), (50, 90), (300, 600)]
    b = [mesh_bytes(*s) for s in sizes]
    assert admit(sizes, 0, sum(b)) == (3, sum(b))
    assert admit(sizes, 0, b[0] + b[1]) == (2, b[0] + b[1])
    assert admit(sizes, 0, b[0] + b[1] + b[2] - 1) == (2, b[0] + b[1])
    # arrival order is kept: a small request behind a large one waits too
    assert admit([(300, 600), (1, 1)], 0, b[0] + 1000) == (1, mesh_bytes(300, 600))  # alone: over budget
    assert admit([(300, 600), (1, 1)], b[0], b[0] + 1000)[0] == 0


def test_admit_memory_held_by_other_slots():
    sizes = [(100, 200)]
    b = mesh_bytes(100, 200)
    assert admit(sizes, 5, b + 5) == (1, b)
    assert admit(sizes, 6, b + 5) == (0, 0)


def test_admit_oversized_request_alone():
    big = [(10 ** 6, 2 * 10 ** 6), (1, 1)]
    b = mesh_bytes(*big[0])
    assert admit(big, 0, b // 2) == (1, b)  # nothing else holds memory: it goes, and fails loudly
    assert admit(big, 1, b // 2) == (0, 0)  # otherwise it waits


def test_poisson_arrivals():
    t = poisson_arrivals(20000, 500.0, seed=3)
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(np.mean(np.diff(t)) - 1 / 500.0) < 0.05 / 500.0
    assert np.array_equal(t, poisson_arrivals(20000, 500.0, seed=3))


def test_carve_meshes_views():
    """A batch's meshes as views of three allocations: exact capacities, no overlap, each triangle segment on a
    16-byte boundary (a multiple of 4 rows of 3 x 4 bytes), empty meshes still one row."""
    torch = pytest.importorskip("torch")
    from miniisosurface_gb300.serve import carve_meshes
    sizes = [(10, 17), (0, 0), (5, 4), (123, 250), (1, 1)]
    for ib in (4, 8):
        ms = carve_meshes(sizes, ib, torch.device("cpu"))
        base = ms[0].tris.data_ptr()
        end_p = end_t = None
        for (v, t), m in zip(sizes, ms):
            assert m.points.shape == (max(v, 1), 3) and m.normals.shape == (max(v, 1), 3)
            assert m.tris.shape == (max(t, 1), 3)
            assert (m.tris.data_ptr() - base) % 16 == 0
            if end_p is not None:
                assert m.points.data_ptr() >= end_p and m.tris.data_ptr() >= end_t
            end_p = m.points.data_ptr() + m.points.numel() * 4
            end_t = m.tris.data_ptr() + m.tris.numel() * ib
            d = m.descriptor()
            assert (d.cap_points, d.cap_tris, d.index_bytes) == (max(v, 1), max(t, 1), ib)


def test_predictor_capacity_rule():
    from miniisosurface_gb300.predictor import Predictor
    p = Predictor(None, margin_t=1.25, v_per_t=0.5, slack=64)
    assert p.capacity(0.0) == (96, 64)
    assert p.capacity(-3.0) == (96, 64)
    assert p.capacity(1000.0) == (int(np.ceil(1314 * 0.5)) + 64, 1314)
