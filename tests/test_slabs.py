"""z-slab decomposition (miniisosurface_gb300.slabs, iso_count_slab, iso_extract_slab).

CPU: the partition and, over two gloo ranks, the count exchange: each rank
holds one slab, takes its counts from the oracle's per-row counts after pass 2,
and the exchanged offsets must be the oracle's own row starts after pass 3 at
the slab boundaries.  GPU: every slab extracted alone, through the C ABI, with
the offsets of the exchange, concatenates to the whole-volume extraction, bit
for bit, for Flying Edges and Marching Cubes.
"""
import os
import socket

import numpy as np
import pytest

import oracle_lib
from miniisosurface_gb300 import slabs


def test_partition_covers_planes():
    for nz in (2, 3, 7, 64, 129):
        for n in (1, 2, 3, 5, 200):
            parts = slabs.partition(nz, n)
            assert parts[0][0] == 0 and parts[-1][1] == nz
            assert all(k0 < k1 for k0, k1 in parts)
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            assert len(parts) == min(n, nz)


def test_data_planes_and_offsets():
    assert slabs.data_planes(0, 4, 10) == (0, 5)
    assert slabs.data_planes(4, 10, 10) == (3, 9)
    assert slabs.data_planes(3, 5, 10) == (2, 6)
    offs, tot = slabs.exclusive_offsets([(5, 7), (0, 0), (3, 1)])
    assert offs == [(0, 0), (5, 7), (5, 7)] and tot == (8, 8)


def _oracle_slab_counts(vol, iso, k0, k1):
    """FE counts of slab [k0, k1) from the oracle's pass-2 row counts."""
    nz, ny, nx = vol.shape
    ge2, tc2, ge3, tc3 = oracle_lib.fe_passes(vol, iso)
    rows = ge2.reshape(nz, ny, 5)
    V = int(rows[k0:k1, :, 2:5].sum())
    T = int(tc2.reshape(nz - 1, ny - 1)[k0:min(k1, nz - 1)].sum())
    ge3 = ge3.reshape(nz, ny, 5)
    tc3 = tc3.reshape(nz - 1, ny - 1)
    want = (int(ge3[k0, 0, 2]), int(tc3[k0, 0]) if k0 < nz - 1 else int(tc2.sum()))
    return (V, T), want


def _exchange_rank(rank, world, port, nz_split, result_dir):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        import miniisosurface_gb300 as M

        vol = M.generate_value_noise((23, 19, 17), 3, 8, seed=5)
        k0, k1 = nz_split[rank]
        (V, T), want = _oracle_slab_counts(vol, 0.05, k0, k1)
        (pv, pt), totals = slabs.exchange_counts(V, T)
        with open(os.path.join(result_dir, "rank%d.txt" % rank), "w") as f:
            f.write("%d %d %d %d %d %d\n" % (pv, pt, want[0], want[1], totals[0], totals[1]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_count_exchange_over_gloo_ranks(built, tmp_path, world):
    import torch.multiprocessing as mp

    split = slabs.partition(17, world)
    mp.spawn(_exchange_rank, args=(world, _free_port(), split, str(tmp_path)), nprocs=world, join=True)
    vol_tot = None
    for r in range(world):
        pv, pt, wv, wt, tv, tt = map(int, (tmp_path / ("rank%d.txt" % r)).read_text().split())
        assert (pv, pt) == (wv, wt), "rank %d offsets %s, oracle row starts %s" % (r, (pv, pt), (wv, wt))
        vol_tot = vol_tot or (tv, tt)
        assert (tv, tt) == vol_tot
    import miniisosurface_gb300 as M

    p, n, t = oracle_lib.fe(M.generate_value_noise((23, 19, 17), 3, 8, seed=5), 0.05)[:3]
    assert vol_tot == (len(p), len(t))


# ---------------------------------------------------------------- GPU
def _mesh_np(mesh):
    return (mesh.points[:mesh.n_points].cpu().numpy(), mesh.normals[:mesh.n_points].cpu().numpy(),
            mesh.tris[:mesh.n_tris].cpu().numpy().astype(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("algo_name", ["FLYING_EDGES", "MARCHING_CUBES"])
def test_multislab_equals_whole_volume(cuda, algo_name):
    import torch
    import miniisosurface_gb300 as M

    algo = getattr(M, algo_name)
    cases = [
        ((64, 40, 37), M.generate_value_noise((64, 40, 37), 3, 16, seed=2), 0.0, (1, 1, 1), (0, 0, 0)),
        ((61, 33, 29), M.generate_blobs((61, 33, 29), 6, seed=3), 0.4, (0.7, 1.3, 0.9), (-2, 1, 5)),
        ((128, 24, 20), M.generate_value_noise((128, 24, 20), 4, 16, seed=4), -0.1, (0.5, 0.5, 2.0), (0, 0, 0)),
    ]
    for dims, vol, iso, sp, org in cases:
        flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
        whole = _mesh_np(M.extract_device(flat, dims, iso, algo, sp, org))
        ref = oracle_lib.fe(vol, iso, sp, org) if algo == M.FLYING_EDGES else oracle_lib.mc(vol, iso, sp, org)
        assert np.array_equal(whole[2], ref[2].astype(np.uint64))
        for n in (1, 2, 3, 5, dims[2]):
            for ib in (4, 8):
                got = _mesh_np(slabs.extract_multislab(flat, dims, iso, algo, n, sp, org, index_bytes=ib))
                assert got[0].shape == whole[0].shape and got[2].shape == whole[2].shape, (dims, n)
                assert np.array_equal(got[2], whole[2]), (dims, n, ib)
                assert np.array_equal(got[0].view(np.uint32), whole[0].view(np.uint32)), (dims, n)
                assert np.array_equal(got[1].view(np.uint32), whole[1].view(np.uint32)), (dims, n)


@pytest.mark.gpu
def test_slab_counts_sum_to_whole(cuda):
    import torch
    import miniisosurface_gb300 as M

    dims = (96, 50, 41)
    vol = M.generate_value_noise(dims, 4, 16, seed=8)
    flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
    for algo in (M.FLYING_EDGES, M.MARCHING_CUBES):
        want = M.count_device(flat, dims, 0.0, algo)
        parts = slabs.partition(dims[2], 4)
        got = [slabs.count_slab(slabs._window(flat, dims, k0, k1), dims, k0, k1, 0.0, algo) for k0, k1 in parts]
        assert tuple(map(sum, zip(*got))) == want


@pytest.mark.gpu
def test_slab_rejects_bad_ranges(cuda):
    import torch
    import miniisosurface_gb300 as M
    from miniisosurface_gb300 import _lib

    dims = (16, 8, 8)
    flat = torch.zeros(16 * 8 * 8, dtype=torch.float32, device="cuda")
    for k0, k1 in ((3, 3), (-1, 2), (5, 9)):
        with pytest.raises(_lib.IsoError):
            slabs.count_slab(flat, dims, k0, k1, 0.0, M.FLYING_EDGES)
