"""Serving loop host logic on CPU: admission by output bytes, Poisson arrivals."""
import numpy as np

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
