"""Allocation-free count entry point (iso_count_device_noalloc), through the C ABI.

Compared with iso_count_device on the same device volumes, two calls in a row
(the second must not see the first one's accumulators), for both algorithms.
The file name keeps it last in collection so it also runs after every other
GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(cuda):
    from miniisosurface_gb300 import _lib

    return _lib.load()


def noalloc_counts(lib, vol_dev, dims, iso, algo):
    import torch
    from miniisosurface_gb300 import api

    out = torch.full((2,), -1, dtype=torch.int64, device=vol_dev.device)
    g = api.make_grid(dims)
    s = torch.cuda.current_stream(vol_dev.device).cuda_stream
    st = lib.iso_count_device_noalloc(algo, C.c_void_p(vol_dev.data_ptr()), C.byref(g), C.c_float(iso),
                                      C.c_void_p(out.data_ptr()), C.c_void_p(s))
    assert st == 0, lib.iso_status_string(st)
    torch.cuda.synchronize()
    return tuple(int(x) for x in out.cpu())


@pytest.mark.parametrize("algo_name", ["FLYING_EDGES", "MARCHING_CUBES"])
def test_noalloc_matches_count_device(lib, algo_name):
    import torch
    import miniisosurface_gb300 as M

    algo = getattr(M, algo_name)
    cases = [
        ((64, 48, 40), M.generate_value_noise((64, 48, 40), 3, 16, seed=3), 0.0),
        ((61, 37, 29), M.generate_blobs((61, 37, 29), 5, seed=4), 0.5),
        ((2300, 3, 4), M.generate_value_noise((2300, 3, 4), 4, 16, seed=5), 0.1),
    ]
    for dims, vol, iso in cases:
        flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
        want = M.count_device(flat, dims, iso, algo)
        first = noalloc_counts(lib, flat, dims, iso, algo)
        second = noalloc_counts(lib, flat, dims, iso, algo)
        assert first == want, (dims, first, want)
        assert second == want, (dims, second, want)


def test_noalloc_dupfree_counts_are_marching_cubes_counts(lib):
    import torch
    import miniisosurface_gb300 as M

    dims = (70, 41, 33)
    flat = torch.from_numpy(M.generate_value_noise(dims, 4, 16, seed=8).reshape(-1)).cuda()
    want = M.count_device(flat, dims, 0.05, M.MARCHING_CUBES)
    assert noalloc_counts(lib, flat, dims, 0.05, M.MC_DUPFREE) == want
    assert noalloc_counts(lib, flat, dims, 0.05, M.MC_DUPFREE) == want


def test_noalloc_empty_and_degenerate(lib):
    import torch
    import miniisosurface_gb300 as M

    for dims in [(8, 9, 10), (1, 5, 5), (5, 1, 5), (5, 5, 1)]:
        flat = torch.ones(dims[0] * dims[1] * dims[2], dtype=torch.float32, device="cuda")
        for algo in (M.FLYING_EDGES, M.MARCHING_CUBES):
            assert noalloc_counts(lib, flat, dims, 0.5, algo) == M.count_device(flat, dims, 0.5, algo) == (0, 0)


def test_noalloc_rejects_grids_beyond_its_scratch(lib):
    import torch
    from miniisosurface_gb300 import _lib, api

    out = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    small = torch.zeros(16, dtype=torch.float32, device="cuda")  # never read: rejected before any launch
    g = api.make_grid((4, 1024, _lib.ISO_NOALLOC_MAX_ROWS // 1024 + 1))
    st = lib.iso_count_device_noalloc(0, C.c_void_p(small.data_ptr()), C.byref(g), C.c_float(0.0),
                                      C.c_void_p(out.data_ptr()), None)
    assert st == _lib.ISO_ERR_TOO_LARGE
    assert b"allocation-free" in lib.iso_status_string(st)
    torch.cuda.synchronize()
    assert out.tolist() == [-1, -1]
    # rows too long for the 32-bit row records: rejected the same way, before any launch
    g = api.make_grid((_lib.ISO_NOALLOC_MAX_ROW_POINTS + 1, 2, 2))
    st = lib.iso_count_device_noalloc(0, C.c_void_p(small.data_ptr()), C.byref(g), C.c_float(0.0),
                                      C.c_void_p(out.data_ptr()), None)
    assert st == _lib.ISO_ERR_TOO_LARGE
    torch.cuda.synchronize()
    assert out.tolist() == [-1, -1]
    # at the limit it runs
    g = api.make_grid((2, 1024, _lib.ISO_NOALLOC_MAX_ROWS // 1024))
    vol = torch.zeros(2 * _lib.ISO_NOALLOC_MAX_ROWS, dtype=torch.float32, device="cuda")
    vol[::2] = 1.0  # every x-edge cut
    st = lib.iso_count_device_noalloc(0, C.c_void_p(vol.data_ptr()), C.byref(g), C.c_float(0.5),
                                      C.c_void_p(out.data_ptr()), None)
    assert st == 0
    torch.cuda.synchronize()
    assert out.tolist()[0] == _lib.ISO_NOALLOC_MAX_ROWS
