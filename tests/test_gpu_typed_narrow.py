"""GPU: 8- and 16-bit samples read as they are (count_narrow.cu, k_vertices
over the sample type) against the same samples converted to float32 first
(iso_ctx_set_narrow(ctx, 0)) and against the oracle on the converted volume,
bit for bit: Flying Edges and Marching Cubes, the three row layouts, isovalues
on a sample value, between two, above and below every sample, 64-bit
indices."""
import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu

TYPES = [(np.int8, 100.0), (np.uint8, 250.0), (np.int16, 8000.0), (np.uint16, 30000.0)]
SHAPES = [(64, 40, 30), (128, 50, 21), (256, 33, 17), (512, 20, 12)]


@pytest.fixture(scope="module")
def M(cuda):
    import miniisosurface_gb300 as M
    return M


def samples(M, dims, dtype, scale, seed):
    f = M.generate_value_noise(dims, 4, 16, seed=seed)
    lo = np.iinfo(dtype).min
    v = np.round(f * scale + (0 if lo < 0 else scale))
    return np.clip(v, lo, np.iinfo(dtype).max).astype(dtype)


def extract(M, vol, dims, iso, algo, narrow, index_bytes=4):
    import torch
    from miniisosurface_gb300 import _lib

    ctx = M.default_context(0)
    _lib.check(_lib.load().iso_ctx_set_narrow(ctx.handle, 1 if narrow else 0), ctx.handle)
    try:
        dv = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).cuda()
        m = M.extract_device(dv, dims, iso, algo, index_bytes=index_bytes, ctx=ctx)
        torch.cuda.synchronize()
        return (m.points[: m.n_points].cpu().numpy(), m.normals[: m.n_points].cpu().numpy(),
                m.tris[: m.n_tris].cpu().numpy().astype(np.uint64))
    finally:
        _lib.load().iso_ctx_set_narrow(ctx.handle, 1)


def same(a, b, what):
    assert a[0].shape == b[0].shape and a[2].shape == b[2].shape, what
    assert np.array_equal(a[2], b[2]), what
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)), what
    assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), what


@pytest.mark.parametrize("dtype,scale", TYPES)
@pytest.mark.parametrize("dims", SHAPES)
def test_narrow_equals_converted(M, dtype, scale, dims):
    if dims[0] * np.dtype(dtype).itemsize % 16:
        pytest.skip("rows not a multiple of 16 bytes: the converted path")
    vol = samples(M, dims, dtype, scale, seed=dims[0])
    mid = float(np.median(vol))
    for algo in (M.FLYING_EDGES, M.MARCHING_CUBES):
        for iso in (mid, mid + 0.5, mid - 0.25):  # on a sample value (ties), between two, just below one
            a = extract(M, vol, dims, iso, algo, True)
            b = extract(M, vol, dims, iso, algo, False)
            same(a, b, "%s %s algo %d iso %r" % (np.dtype(dtype).name, dims, algo, iso))


@pytest.mark.parametrize("dtype,scale", TYPES)
def test_narrow_against_oracle(M, dtype, scale):
    dims = (64, 36, 25)
    vol = samples(M, dims, dtype, scale, seed=11)
    iso = float(np.percentile(vol, 40))
    f = vol.astype(np.float32)
    same(extract(M, vol, dims, iso, M.FLYING_EDGES, True), oracle_lib.fe(f, iso)[:3], "FE vs oracle")
    same(extract(M, vol, dims, iso, M.MARCHING_CUBES, True), oracle_lib.mc(f, iso)[:3], "MC vs oracle")
    same(extract(M, vol, dims, iso, M.FLYING_EDGES, True, index_bytes=8), oracle_lib.fe(f, iso)[:3],
         "FE 64-bit indices")


def test_narrow_isovalues_outside_the_samples(M):
    dims = (64, 20, 10)
    for dtype, scale in TYPES:
        vol = samples(M, dims, dtype, scale, seed=3)
        info = np.iinfo(dtype)
        for iso in (float(info.max) + 1.0, float(info.min) - 0.5, 1e30, -1e30):
            a = extract(M, vol, dims, iso, M.FLYING_EDGES, True)
            assert a[0].shape == (0, 3) and a[2].shape == (0, 3), (np.dtype(dtype).name, iso)
        # every sample at or above the smallest: no surface either
        a = extract(M, vol, dims, float(info.min), M.FLYING_EDGES, True)
        assert a[2].shape == (0, 3)
