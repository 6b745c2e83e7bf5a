"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Bar: triangle count, connectivity and vertex numbering bit-exact; points and
normals bit-identical float32 (the kernels evaluate the reference's float
formulas in the same order with no FMA contraction; the stated tolerance of
2 ulp is never needed).
"""
import ctypes as C
import os
from pathlib import Path

import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu

POS_ULP_TOL = 0  # measured: 0 ulp; the contract allows 2


def ulp_diff(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-2**31) - ia, ia)
    ib = np.where(ib < 0, np.int64(-2**31) - ib, ib)
    return np.abs(ia - ib)


def assert_same_mesh(got, ref, what=""):
    p, n, t = got
    rp, rn, rt = ref[:3]
    assert p.shape == rp.shape, "%s vertex count %s vs %s" % (what, p.shape, rp.shape)
    assert t.shape == rt.shape, "%s triangle count %s vs %s" % (what, t.shape, rt.shape)
    assert np.array_equal(t.astype(np.uint64), rt.astype(np.uint64)), "%s connectivity differs" % what
    if p.size:
        assert ulp_diff(p, rp).max() <= POS_ULP_TOL, "%s points differ" % what
        assert ulp_diff(n, rn).max() <= POS_ULP_TOL, "%s normals differ" % what


def gpu_extract(M, vol, iso, algo, spacing=(1, 1, 1), origin=(0, 0, 0), index_bytes=4, offset=0):
    import torch

    nz, ny, nx = vol.shape
    flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
    if offset:
        buf = torch.empty(flat.numel() + offset, dtype=torch.float32, device="cuda")
        buf[offset:] = flat
        flat = buf[offset:]
    mesh = M.extract_device(flat, (nx, ny, nz), iso, algo, spacing, origin, index_bytes=index_bytes)
    torch.cuda.synchronize()
    return (mesh.points[: mesh.n_points].cpu().numpy(), mesh.normals[: mesh.n_points].cpu().numpy(),
            mesh.tris[: mesh.n_tris].cpu().numpy().astype(np.uint64))


def both(M, vol, iso, spacing=(1, 1, 1), origin=(0, 0, 0), **kw):
    got = gpu_extract(M, vol, iso, M.FLYING_EDGES, spacing, origin, **kw)
    assert_same_mesh(got, oracle_lib.fe(vol, iso, spacing, origin), "FE")
    got = gpu_extract(M, vol, iso, M.MARCHING_CUBES, spacing, origin, **kw)
    assert_same_mesh(got, oracle_lib.mc(vol, iso, spacing, origin), "MC")


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def test_blobs_config0_128(M):
    vol = M.generate_blobs((128, 128, 128), 8, seed=0)
    both(M, vol, 0.5)


def test_blobs_spacing_origin(M):
    vol = M.generate_blobs((40, 33, 27), 8, seed=3)
    both(M, vol, 0.5, (0.1, 0.37, 1.3), (-2.5, 0.3, 7.1))
    both(M, vol, 0.31, (2.0, 0.5, 0.03125), (1e3, -7.25, 0.0))


def test_noise_nonaligned_rows(M):
    vol = M.generate_value_noise((61, 47, 35), 4, 16, seed=5)
    both(M, vol, 0.0)
    both(M, vol, 0.2, (0.3, 0.3, 0.3), (0.1, 0.2, 0.3))


def test_unaligned_volume_pointer(M):
    vol = M.generate_value_noise((64, 20, 20), 3, 8, seed=9)
    both(M, vol, 0.05, offset=1)


def test_wide_rows_multi_chunk(M):
    # nx > 32*32 points: rows span several 32-word chunks
    vol = M.generate_value_noise((1500, 5, 4), 4, 16, seed=11)
    both(M, vol, 0.0)
    vol = M.generate_value_noise((1029, 3, 3), 4, 8, seed=12)
    both(M, vol, 0.1)
    # nx > 64*32 points: the chunked count kernel
    vol = M.generate_value_noise((2300, 4, 3), 4, 16, seed=13)
    both(M, vol, 0.0)
    vol = M.generate_value_noise((4099, 2, 3), 4, 8, seed=14)
    both(M, vol, -0.05)


@pytest.mark.parametrize("dims", [(600, 9, 7), (1000, 7, 6), (1024, 5, 5), (513, 10, 6), (557, 8, 6),
                                  (1023, 6, 5)])
def test_rows_of_17_to_32_words(M, dims):
    """Rows of 513-1024 points: one grid row per warp in pass 4 (Flying Edges
    vertices through the per-axis queues) and in the bulk-copy count pass (rows
    a multiple of 4 points long, 1024 points, and not: 513, 557, 1023)."""
    vol = M.generate_value_noise(dims, 4, 16, seed=sum(dims))
    both(M, vol, 0.0)


@pytest.mark.parametrize("dims", [(8, 6, 1500), (20, 3, 4000)])
def test_tall_grids(M, dims):
    """Thousands of planes: many plane runs of work items, plane numbers well
    past the first bytes of the vertex records."""
    rng = np.random.default_rng(dims[2])
    vol = rng.standard_normal(dims[::-1]).astype(np.float32)
    both(M, vol, 0.1, (1.0, 0.5, 0.25), (0.0, 1.0, -3.0))


@pytest.mark.parametrize("nx", [124, 127, 128, 129, 132, 251, 252, 255, 256, 257, 260, 506, 508, 511, 512])
def test_row_width_boundaries(M, nx):
    """Rows at the edges of the kernel choices: up to 4 words the count and
    generate kernels put eight rows in a warp (128 points: every lane's word
    full), up to 8 words four (256: full), from 9 to 16 words two (512:
    full); 13 rows leave the last group of rows short.  Widths that are not a
    multiple of 4 points put the rows of a plane at every offset from a
    16-byte boundary in the count kernel's plane copies."""
    vol = M.generate_value_noise((nx, 13, 11), 3, 16, seed=nx)
    both(M, vol, 0.0)
    rng = np.random.default_rng(nx)
    vol = rng.standard_normal((9, 13, nx)).astype(np.float32)
    both(M, vol, 0.2, (0.5, 1.5, 0.75), (1.0, -2.0, 0.5))


@pytest.mark.parametrize("dims", [(2, 2, 2), (2, 9, 5), (3, 2, 7), (33, 2, 2), (5, 6, 2), (31, 32, 33), (32, 17, 9),
                                  (65, 3, 4), (97, 11, 13)])
def test_random_small(M, dims):
    rng = np.random.default_rng(sum(dims))
    nx, ny, nz = dims
    for trial in range(3):
        vol = rng.standard_normal((nz, ny, nx)).astype(np.float32)
        iso = float(rng.uniform(-0.5, 0.5))
        both(M, vol, iso, tuple(rng.uniform(0.1, 2.0, 3)), tuple(rng.uniform(-5, 5, 3)))


def test_ties_equal_isovalue(M):
    # integer field, isovalue hit exactly: classification uses >=
    rng = np.random.default_rng(1)
    vol = rng.integers(-2, 3, size=(13, 11, 17)).astype(np.float32)
    for iso in (-1.0, 0.0, 1.0, 2.0):
        both(M, vol, iso)


def test_all_256_cube_cases(M):
    for c in range(256):
        vol = np.zeros((2, 2, 2), np.float32)
        corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        for v, (i, j, k) in enumerate(corner):
            vol[k, j, i] = 1.0 + 0.25 * v if (c >> v) & 1 else -1.0 - 0.125 * v
        both(M, vol, 0.0)


def test_empty_meshes(M):
    vol = np.ones((8, 9, 10), np.float32)
    for iso in (0.5, 2.0):          # all above / all below
        both(M, vol, iso)
    for dims in [(1, 5, 5), (5, 1, 5), (5, 5, 1)]:   # degenerate grids
        vol = np.random.default_rng(0).standard_normal(dims[::-1]).astype(np.float32)
        got = gpu_extract(M, vol, 0.0, M.FLYING_EDGES)
        assert got[0].shape == (0, 3) and got[2].shape == (0, 3)


def test_index_widths_agree(M):
    vol = M.generate_value_noise((48, 40, 36), 4, 16, seed=2)
    for algo in (M.FLYING_EDGES, M.MARCHING_CUBES):
        a = gpu_extract(M, vol, 0.0, algo, index_bytes=4)
        b = gpu_extract(M, vol, 0.0, algo, index_bytes=8)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_host_entry_point(M):
    vol = M.generate_blobs((50, 41, 37), 8, seed=4)
    img = M.Image3D.from_array(vol, (0.5, 0.5, 2.0), (1.0, -1.0, 0.5))
    for algo, ref in ((M.FLYING_EDGES, oracle_lib.fe), (M.MARCHING_CUBES, oracle_lib.mc)):
        m = M.extract(img, 0.5, algo)
        assert_same_mesh((m.points, m.normals, m.triangles), ref(vol, 0.5, img.spacing, img.zeroPos))
    m = M.MarchingCubes(img, 0.5)
    assert_same_mesh((m.points, m.normals, m.triangles), oracle_lib.mc(vol, 0.5, img.spacing, img.zeroPos))


def test_host_entry_point_streamed(M):
    """Grids of 128 planes and more take the streamed host path (slabs copied into
    three device windows, counted, generated and copied back on overlapping
    streams); 450 planes reuse every window twice."""
    cases = [((70, 45, 200), M.generate_value_noise((70, 45, 200), 3, 16, seed=6), 0.0, (1.0, 1.0, 1.0)),
             ((64, 33, 130), M.generate_blobs((64, 33, 130), 7, seed=7), 0.45, (0.75, 1.5, 0.5)),
             ((40, 30, 450), M.generate_value_noise((40, 30, 450), 3, 8, seed=9), 0.1, (1.0, 0.5, 1.0))]
    for dims, vol, iso, sp in cases:
        img = M.Image3D.from_array(vol, sp, (2.0, -1.0, 0.25))
        for algo, ref in ((M.FLYING_EDGES, oracle_lib.fe), (M.MARCHING_CUBES, oracle_lib.mc)):
            want = ref(vol, iso, img.spacing, img.zeroPos)
            for ib in (4, 8):
                m = M.extract(img, iso, algo, index_bytes=ib)
                assert_same_mesh((m.points, m.normals, m.triangles), want, "streamed %s ib %d" % (dims, ib))


def test_host_entry_point_streamed_pinned(M):
    """Streamed host path into pinned output buffers (the bench's end-to-end
    case), each slab's part of the mesh at its offset in them; buffers that
    start 4 bytes past a 16-byte boundary too."""
    import torch
    from miniisosurface_gb300 import _lib

    lib = _lib.load()
    ctx = M.Context(0)
    dims = (70, 45, 200)
    vol = M.generate_value_noise(dims, 3, 16, seed=6)
    img = M.Image3D.from_array(vol, (1.0, 0.5, 1.0), (2.0, -1.0, 0.25))
    g = img.grid()
    for algo, ref in ((M.FLYING_EDGES, oracle_lib.fe), (M.MARCHING_CUBES, oracle_lib.mc)):
        want = ref(vol, 0.0, img.spacing, img.zeroPos)
        V, T = want[0].shape[0], want[2].shape[0]
        for ib, shift in ((4, 0), (8, 0), (4, 1), (8, 1)):
            it = torch.int32 if ib == 4 else torch.int64
            # shift words of padding at the front of each buffer
            hp = torch.zeros(3 * V + shift, dtype=torch.float32).pin_memory()
            hn = torch.zeros(3 * V + shift, dtype=torch.float32).pin_memory()
            ht = torch.zeros(3 * T * ib // 4 + shift, dtype=torch.int32).pin_memory()
            m = _lib.IsoMesh()
            m.points, m.normals = hp.data_ptr() + 4 * shift, hn.data_ptr() + 4 * shift
            m.tris = ht.data_ptr() + 4 * shift
            m.index_bytes, m.cap_points, m.cap_tris = ib, V, T
            st = lib.iso_extract_host(ctx.handle, M.api._algo(algo), img.data.ctypes.data, C.byref(g), C.c_float(0.0),
                                      C.byref(m), None)
            _lib.check(st, ctx.handle)
            assert (m.n_points, m.n_tris) == (V, T)
            p = hp.numpy()[shift:].reshape(V, 3)
            n = hn.numpy()[shift:].reshape(V, 3)
            tr = ht.numpy()[shift:].view(np.int32 if ib == 4 else np.int64).reshape(T, 3).astype(np.uint64)
            assert_same_mesh((p, n, tr), want, "pinned algo %s ib %d shift %d" % (algo, ib, shift))


def test_mc_dupfree_matches_oracle(M):
    """ISO_MC_DUPFREE: the serial MC mesh with vertices in global-edge-index
    order (marchingCubes/openmpDupFree with one section), bit for bit."""
    import torch

    cases = [((128, 128, 128), M.generate_blobs((128, 128, 128), 8, seed=0), 0.5, (1, 1, 1), (0, 0, 0)),
             ((61, 37, 29), M.generate_value_noise((61, 37, 29), 3, 8, seed=2), 0.05, (0.3, 1.7, 0.9), (3, -2, 1)),
             ((33, 2, 2), np.random.default_rng(4).standard_normal((2, 2, 33)).astype(np.float32), 0.0, (1, 1, 1),
              (0, 0, 0)),
             ((1000, 5, 4), M.generate_value_noise((1000, 5, 4), 4, 16, seed=3), 0.0, (1, 1, 1), (0, 0, 0))]
    for dims, vol, iso, sp, org in cases:
        want = oracle_lib.mc_dupfree(vol, iso, sp, org)
        for ib in (4, 8):
            got = gpu_extract(M, vol, iso, M.MC_DUPFREE, sp, org, index_bytes=ib)
            assert_same_mesh(got, want, "dupfree %s" % (dims,))
        img = M.Image3D.from_array(vol, sp, org)
        m = M.extract(img, iso, M.MC_DUPFREE)
        assert_same_mesh((m.points, m.normals, m.triangles), want, "dupfree host %s" % (dims,))
        flat = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
        assert M.count_device(flat, dims, iso, M.MC_DUPFREE) == (len(want[0]), len(want[2]))


@pytest.mark.parametrize("dtype", ["int8", "uint8", "int16", "uint16", "int32", "float64"])
def test_typed_volumes(M, dtype):
    """Volumes of the reference's other sample types: converted to float32 on
    the device (host and device entry points, streamed and not), the same mesh
    as the oracle on volume.astype(float32)."""
    import torch

    rng = np.random.default_rng(len(dtype))
    info = np.iinfo(dtype) if dtype not in ("float64",) else None
    for dims in ((45, 33, 28), (40, 30, 200)):
        noise = M.generate_value_noise(dims, 3, 8, seed=5)
        if info is not None:
            lo, hi = int(info.min), int(info.max)
            scaled = np.round((noise.astype(np.float64) + 1.5) / 3.0 * (hi - lo) + lo)
            vol = np.clip(scaled.astype(np.int64), lo, hi).astype(dtype)
            iso = float(np.float32((lo + hi) / 2 + 0.5))
        else:
            vol = (noise.astype(np.float64) * 1.000000123)
            iso = 0.01
        ref_vol = vol.astype(np.float32)
        for algo, ref in ((M.FLYING_EDGES, oracle_lib.fe), (M.MARCHING_CUBES, oracle_lib.mc)):
            want = ref(ref_vol, iso)
            m = M.extract_typed(vol, iso, algo)
            assert_same_mesh((m.points, m.normals, m.triangles), want, "host %s %s" % (dtype, dims))
            dev = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
            mesh = M.extract_device(dev, dims, iso, algo)
            got = (mesh.points[:mesh.n_points].cpu().numpy(), mesh.normals[:mesh.n_points].cpu().numpy(),
                   mesh.tris[:mesh.n_tris].cpu().numpy().astype(np.uint64))
            assert_same_mesh(got, want, "device %s %s" % (dtype, dims))


def test_fe_pass_by_pass_state(M):
    """gridEdges (xl, xr, xstart, ystart, zstart) and triCounter after pass 2
    and pass 3 equal the reference algorithm's state."""
    vol = M.generate_value_noise((45, 30, 22), 4, 16, seed=8)
    img = M.Image3D.from_array(vol)
    fe = M.FlyingEdgesAlgorithm(img, 0.1)
    fe.pass1()
    fe.pass2()
    ge2, tc2 = fe.gridEdges()
    fe.pass3()
    ge3, tc3 = fe.gridEdges()
    fe.pass4()
    mesh = fe.moveOutput()
    rge2, rtc2, rge3, rtc3 = oracle_lib.fe_passes(vol, 0.1)
    assert np.array_equal(ge2, rge2)
    assert np.array_equal(tc2, rtc2)
    assert np.array_equal(ge3, rge3)
    assert np.array_equal(tc3, rtc3)
    assert_same_mesh((mesh.points, mesh.normals, mesh.triangles), oracle_lib.fe(vol, 0.1))


def test_capacity_error_reports_sizes(M):
    import torch
    from miniisosurface_gb300 import _lib

    vol = M.generate_blobs((32, 32, 32), 8, seed=1)
    flat = torch.from_numpy(vol.reshape(-1)).cuda()
    small = M.DeviceMesh(10, 10, 4)
    m = small.descriptor()
    g = M.make_grid((32, 32, 32))
    lib = _lib.load()
    ctx = M.default_context(0)
    st = lib.iso_extract_device(ctx.handle, M.FLYING_EDGES, flat.data_ptr(), C.byref(g), C.c_float(0.5),
                                C.byref(m), None)
    assert st == _lib.ISO_ERR_CAPACITY
    rp, rn, rt, _ = oracle_lib.fe(vol, 0.5)
    assert (m.n_points, m.n_tris) == (rp.shape[0], rt.shape[0])
    nv, nt = M.count_device(flat, (32, 32, 32), 0.5)
    assert (nv, nt) == (rp.shape[0], rt.shape[0])


def _fp64_report(name, err):
    """Print the case's FP64 error; with MINIISO_REPORT_DIR set (an existing folder), also append it to
    fp64_error.jsonl there."""
    import json

    out = os.environ.get("MINIISO_REPORT_DIR")
    if out and Path(out).is_dir():
        with open(Path(out) / "fp64_error.jsonl", "a") as f:
            f.write(json.dumps({"case": name, **err}) + "\n")
    print(name, err)


def test_fp64_interpolation_error(M):
    """Max error of the float32 points/normals against the same formulas in
    double precision (reported; bounded by a few float32 ulps of the field)."""
    vol = M.generate_blobs((64, 64, 64), 8, seed=2)
    sp, org = (0.7, 0.3, 1.1), (-1.0, 2.0, 0.5)
    p, n, t = gpu_extract(M, vol, 0.5, M.FLYING_EDGES, sp, org)
    _, _, _, eov = oracle_lib.fe(vol, 0.5, sp, org)
    err = oracle_lib.fp64_error(vol, 0.5, p, n, eov, sp, org)
    _fp64_report("blobs64_spacing", err)
    eps = np.finfo(np.float32).eps
    assert err["points"]["max_rel"] <= 8 * eps
    assert err["normals"]["max_rel"] <= 64 * eps


def test_fp64_error_config0(M):
    """The FP64 error on the 128^3 Gaussian-blob volume at isovalue 0.5."""
    vol = M.generate_blobs((128, 128, 128), 8, seed=0)
    p, n, t = gpu_extract(M, vol, 0.5, M.FLYING_EDGES)
    _, _, _, eov = oracle_lib.fe(vol, 0.5)
    err = oracle_lib.fp64_error(vol, 0.5, p, n, eov)
    _fp64_report("blobs128_iso0.5", err)
    eps = np.finfo(np.float32).eps
    assert err["points"]["max_rel"] <= 8 * eps
    assert err["normals"]["max_rel"] <= 64 * eps


def test_noise_512_bitexact(M):
    """The bench workload: 512^3 value noise at isovalue 0, FE and MC."""
    vol = M.generate_value_noise((512, 512, 512), 4, 64, seed=1)
    got = gpu_extract(M, vol, 0.0, M.FLYING_EDGES)
    ref = oracle_lib.fe(vol, 0.0, nthreads=os.cpu_count())
    assert_same_mesh(got, ref, "FE 512")
    _fp64_report("noise512_iso0", oracle_lib.fp64_error(vol, 0.0, got[0], got[1], ref[3]))
    del got, ref
    got = gpu_extract(M, vol, 0.0, M.MARCHING_CUBES)
    ref = oracle_lib.mc(vol, 0.0)
    assert_same_mesh(got, ref, "MC 512")


def test_mc_triangles_into_unaligned_buffer(M):
    """Marching Cubes over rows of up to 16 words writes FE-id triangles and remaps them in place: a triangle
    buffer 4 bytes past a 16-byte boundary takes the remap's one-by-one path, with the same mesh."""
    import torch
    vol = M.generate_value_noise((61, 47, 35), 4, 16, seed=5)
    ref = oracle_lib.mc(vol, 0.0)
    V, T = ref[0].shape[0], ref[2].shape[0]
    dv = torch.from_numpy(vol.reshape(-1)).cuda()
    for ib, dt in ((4, torch.int32), (8, torch.int64)):
        m = M.DeviceMesh(V, T, ib)
        buf = torch.empty(3 * T + 1, dtype=dt, device="cuda")
        m.tris = buf[1:].view(T, 3)
        got = M.extract_device(dv, (61, 47, 35), 0.0, M.MARCHING_CUBES, out=m, index_bytes=ib)
        torch.cuda.synchronize()
        assert got is m
        assert_same_mesh((m.points[:V].cpu().numpy(), m.normals[:V].cpu().numpy(),
                          m.tris[:T].cpu().numpy().astype(np.uint64)), ref, "MC unaligned tris ib %d" % ib)
