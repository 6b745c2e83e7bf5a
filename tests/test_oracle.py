"""CPU: the oracle pinned against the reference.

1. Golden fixtures (tests/golden/golden.json), produced by running the
   reference programs compiled from the miniIsosurface sources.
2. When oracle/_ref/ exists (built here from the reference sources): the
   reference programs themselves on further seeded volumes, including the
   OpenMP Flying Edges variant.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle_lib

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(b):
    return hashlib.sha256(b).hexdigest()


def golden_cases():
    return json.loads((GOLDEN / "golden.json").read_text())


def golden_volume(rec):
    import miniisosurface_gb300 as M

    if "npy" in rec:
        vol = np.load(GOLDEN / rec["npy"])
    else:
        g = rec["gen"]
        if g["kind"] == "blobs":
            vol = M.generate_blobs(g["dims"], g["nblobs"], g["seed"])
        else:
            vol = M.generate_value_noise(g["dims"], g["octaves"], g["period"], g["seed"])
    assert sha(np.ascontiguousarray(vol, "<f4").tobytes()) == rec["volume_sha256"], "input volume drifted"
    return vol


def digest(p, n, t):
    return dict(n_points=int(p.shape[0]), n_tris=int(t.shape[0]),
                points=sha(np.ascontiguousarray(p, "<f4").tobytes()),
                normals=sha(np.ascontiguousarray(n, "<f4").tobytes()),
                tris=sha(np.ascontiguousarray(t, "<u8").tobytes()))


@pytest.mark.parametrize("rec", golden_cases(), ids=lambda r: r["name"])
def test_oracle_matches_golden(built, rec):
    vol = golden_volume(rec)
    for algo, fn in (("fe", oracle_lib.fe), ("mc", oracle_lib.mc)):
        p, n, t, _ = fn(vol, rec["iso"], rec["spacing"], rec["origin"])
        d = digest(p, n, t)
        for key in d:
            assert d[key] == rec[algo][key], "%s %s %s" % (rec["name"], algo, key)


@pytest.mark.parametrize("rec", golden_cases(), ids=lambda r: r["name"])
def test_mesh_writer_byte_identical_to_reference(built, rec, tmp_path):
    """util::saveTriangleMesh layout, byte for byte (sha256 of the reference file)."""
    import miniisosurface_gb300 as M

    vol = golden_volume(rec)
    for algo, fn in (("fe", oracle_lib.fe), ("mc", oracle_lib.mc)):
        p, n, t, _ = fn(vol, rec["iso"], rec["spacing"], rec["origin"])
        path = tmp_path / ("%s.vtk" % algo)
        M.saveTriangleMesh(M.TriangleMesh(p, n, t), str(path))
        assert sha(path.read_bytes()) == rec[algo]["vtk"]


def test_openmp_oracle_equals_serial(built):
    import miniisosurface_gb300 as M

    vol = M.generate_value_noise((70, 60, 50), 4, 16, seed=3)
    a = oracle_lib.fe(vol, 0.0, nthreads=1)
    b = oracle_lib.fe(vol, 0.0, nthreads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


needs_ref = pytest.mark.skipif(not oracle_lib.ref_available(), reason="reference programs not built here")


@needs_ref
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_vs_reference_programs(built, seed):
    import miniisosurface_gb300 as M

    rng = np.random.default_rng(seed)
    dims = tuple(int(x) for x in rng.integers(2, 40, 3))
    vol = M.generate_value_noise(dims, 4, 8, seed=seed)
    iso = float(rng.uniform(-0.3, 0.3))
    # float32 values: the VTK header text then parses back to the same floats
    sp = tuple(float(np.float32(x)) for x in rng.uniform(0.1, 3, 3))
    org = tuple(float(np.float32(x)) for x in rng.uniform(-10, 10, 3))
    for prog, fn in (("flyingEdgesSerial", oracle_lib.fe), ("mcSerial", oracle_lib.mc),
                     ("flyingEdgesOpenMP", oracle_lib.fe)):
        rp, rn, rt, _, _ = oracle_lib.run_ref(prog, vol, iso, sp, org, threads=3)
        p, n, t, _ = fn(vol, iso, sp, org)
        assert np.array_equal(rt, t), prog
        assert np.array_equal(rp.view(np.uint32), p.view(np.uint32)), prog
        assert np.array_equal(rn.view(np.uint32), n.view(np.uint32)), prog


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-2**31) - ia, ia)
    ib = np.where(ib < 0, np.int64(-2**31) - ib, ib)
    return np.abs(ia - ib)


@pytest.mark.skipif(not oracle_lib.ref_available("mcOpenMPDupFree"), reason="reference programs not built here")
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_dupfree_oracle_vs_reference_program(built, seed):
    """marchingCubes/openmpDupFree: with one thread (one section) its mesh is
    the oracle's global-edge-index order bit for bit; with four sections the
    vertices are the same in the same order, a seam vertex computed by the
    cell on either side of the seam (positions within 2 ulp, normals equal),
    and the triangles the same set."""
    import miniisosurface_gb300 as M

    rng = np.random.default_rng(100 + seed)
    dims = tuple(int(x) for x in rng.integers(8, 40, 3))
    vol = M.generate_value_noise(dims, 4, 8, seed=seed)
    iso = float(rng.uniform(-0.3, 0.3))
    sp = tuple(float(np.float32(x)) for x in rng.uniform(0.1, 3, 3))
    org = tuple(float(np.float32(x)) for x in rng.uniform(-10, 10, 3))
    p, n, t, eov = oracle_lib.mc_dupfree(vol, iso, sp, org)
    assert np.all(np.diff(eov.astype(np.int64)) > 0)  # strictly increasing global edge index
    rp, rn, rt, _, _ = oracle_lib.run_ref("mcOpenMPDupFree", vol, iso, sp, org, threads=1)
    assert np.array_equal(rt, t)
    assert np.array_equal(rp.view(np.uint32), p.view(np.uint32))
    assert np.array_equal(rn.view(np.uint32), n.view(np.uint32))
    rp4, rn4, rt4, _, _ = oracle_lib.run_ref("mcOpenMPDupFree", vol, iso, sp, org, threads=4)
    assert rp4.shape == p.shape
    assert _ulps(rp4, p).max() <= 2
    assert np.array_equal(rn4.view(np.uint32), n.view(np.uint32))
    key = lambda a: a[np.lexsort(a.T[::-1])]
    assert np.array_equal(key(rt4), key(t.astype(rt4.dtype)))


@needs_ref
def test_product_image_writer_readable_by_reference(built, tmp_path):
    """A volume written by iso_vtk_write_image loads in the reference loader."""
    import subprocess

    import miniisosurface_gb300 as M

    vol = M.generate_blobs((20, 18, 16), 8, seed=2)
    img = M.Image3D.from_array(vol, (0.5, 1.5, 2.0), (1, 2, 3))
    path = tmp_path / "v.vtk"
    M.saveImage(img, str(path))
    out = tmp_path / "m.vtk"
    subprocess.run([str(oracle_lib.REF_DIR / "flyingEdgesSerial"), "-i", str(path), "-o", str(out), "-v", "0.5",
                    "-y", str(tmp_path / "y.yaml")], check=True, capture_output=True)
    rp, rn, rt = oracle_lib.read_polydata(out)
    p, n, t, _ = oracle_lib.fe(vol, 0.5, img.spacing, img.zeroPos)
    assert np.array_equal(rt, t) and np.array_equal(rp, p) and np.array_equal(rn, n)
    back = M.loadImage(str(path))
    assert back.dims == img.dims and np.array_equal(back.data, img.data)
    assert back.spacing == img.spacing and back.zeroPos == img.zeroPos


def test_oracle_generators_match_golden_and_product(built):
    """The oracle's own volume generator (used by the CPU arm of the bench, which
    must not load the product library) gives the pinned volume digests and the
    product generator's volumes bit for bit."""
    import hashlib
    import json

    import miniisosurface_gb300 as M

    golden = {c["name"]: c for c in golden_cases()}
    c0 = golden["blobs128_config0"]
    vol = oracle_lib.generate_blobs(c0["gen"]["dims"], c0["gen"]["nblobs"], c0["gen"]["seed"])
    assert hashlib.sha256(np.ascontiguousarray(vol, "<f4").tobytes()).hexdigest() == c0["volume_sha256"]
    c1 = golden["noise96x80x72"]
    g = c1["gen"]
    vol = oracle_lib.generate_value_noise(g["dims"], g["octaves"], g["period"], g["seed"])
    assert hashlib.sha256(np.ascontiguousarray(vol, "<f4").tobytes()).hexdigest() == c1["volume_sha256"]
    for dims in ((33, 20, 17), (5, 64, 3)):
        assert np.array_equal(oracle_lib.generate_value_noise(dims, 3, 8, 9), M.generate_value_noise(dims, 3, 8, seed=9))
        assert np.array_equal(oracle_lib.generate_blobs(dims, 5, 11), M.generate_blobs(dims, 5, seed=11))


def _tri_corners(p, t):
    """Triangles as rows of their 9 corner coordinates (bit patterns), sorted."""
    c = p[t.astype(np.int64)].reshape(len(t), 9).view(np.uint32)
    return c[np.lexsort(c.T[::-1])]


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_mc_openmp_port_sections(built, threads):
    """The OpenMP Marching Cubes port: one thread is the serial mesh; with more
    threads each z-section numbers its own vertices (seam vertices repeated),
    and the triangles are the serial ones, corner for corner."""
    vol = oracle_lib.generate_value_noise((30, 26, 40), 4, 8, 3)
    sp, org = (0.5, 1.5, 0.75), (1.0, -2.0, 0.5)
    sp_ = oracle_lib.mc(vol, 0.1, sp, org)
    om = oracle_lib.mc_openmp(vol, 0.1, sp, org, nthreads=threads)
    if threads == 1:
        for x, y in zip(sp_, om):
            assert np.array_equal(x, y)
    else:
        assert om[0].shape[0] > sp_[0].shape[0]  # vertices on the seams appear once per section
        assert om[2].shape == sp_[2].shape
        assert np.array_equal(_tri_corners(om[0], om[2]), _tri_corners(sp_[0], sp_[2]))
        assert len(np.unique(om[3])) == sp_[0].shape[0]  # the same edges


@pytest.mark.skipif(not oracle_lib.ref_available("mcOpenMP"), reason="reference programs not built here")
@pytest.mark.parametrize("threads", [1, 4])
def test_mc_openmp_port_vs_reference_program(built, threads):
    """Against marchingCubes/openmp itself: the same vertex count (seams
    included) and the same triangles corner for corner; with one thread the
    same mesh bit for bit (the program appends its threads' meshes in the
    order they finish, so only one thread fixes the order)."""
    vol = oracle_lib.generate_value_noise((34, 29, 37), 4, 8, 5)
    sp, org = (1.25, 0.5, 1.0), (0.0, 3.0, -1.0)
    rp, rn, rt, _, _ = oracle_lib.run_ref("mcOpenMP", vol, 0.05, sp, org, threads=threads)
    p, n, t, _ = oracle_lib.mc_openmp(vol, 0.05, sp, org, nthreads=threads)
    assert rp.shape == p.shape and rt.shape == t.shape
    if threads == 1:
        assert np.array_equal(rt, t)
        assert np.array_equal(rp.view(np.uint32), p.view(np.uint32))
        assert np.array_equal(rn.view(np.uint32), n.view(np.uint32))
    else:
        assert np.array_equal(_tri_corners(rp, rt), _tri_corners(p, t))
