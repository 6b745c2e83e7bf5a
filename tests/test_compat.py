"""C++ integration headers: include/miniiso_fe.hpp (drop-in FlyingEdgesAlgorithm)
and include/miniiso_mc.hpp (MarchingCubes body).

CPU: the reference's own flyingEdges/serial/main.cpp compiles and links
unchanged against the shim (when a reference checkout is present), and the
shim check program compiles.  GPU: the shim check program, run through both
headers, gives the oracle's meshes bit for bit.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib

ROOT = Path(__file__).resolve().parents[1]
REF = oracle_lib.REFERENCE
COMPAT = ROOT / "tests" / "compat"


def lib_dir():
    from miniisosurface_gb300 import builder

    return builder.library_path().parent


def run(cmd):
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    assert res.returncode == 0, "%s\n%s%s" % (" ".join(map(str, cmd)), res.stdout, res.stderr)
    return res.stdout


def build_shim_check(out):
    d = lib_dir()
    run(["g++", "-O2", "-std=c++14", "-I", ROOT / "include", "-I", COMPAT / "standin", COMPAT / "shim_check.cpp",
         "-o", out, "-L", d, "-lminiiso", "-Wl,-rpath," + str(d)])
    return out


def test_shim_check_compiles(built, tmp_path):
    assert build_shim_check(tmp_path / "shim_check").exists()


@pytest.mark.skipif(not (REF / "flyingEdges" / "serial" / "main.cpp").exists(), reason="no reference checkout")
def test_reference_main_builds_against_shim(built, tmp_path):
    fe = REF / "flyingEdges"
    d = lib_dir()
    exe = tmp_path / "flyingEdgesGB300"
    run(["g++", "-O2", "-std=c++11", "-w", "-include", ROOT / "include" / "miniiso_fe.hpp", "-I", ROOT / "include",
         "-I", fe / "util", fe / "serial" / "main.cpp", fe / "util" / "Image3D.cpp", fe / "util" / "Timer.cpp",
         fe / "mantevoCommon" / "YAML_Doc.cpp", fe / "mantevoCommon" / "YAML_Element.cpp", "-o", exe, "-L", d,
         "-lminiiso", "-Wl,-rpath," + str(d)])
    assert exe.exists()
    syms = run(["nm", "-C", "-u", exe])
    assert "iso_fe_pass4" in syms  # the passes come from the library, not from the reference's .cpp


def read_dump(path):
    raw = Path(path).read_bytes()
    V, T = np.frombuffer(raw[:16], np.int64)
    off = 16
    pts = np.frombuffer(raw[off:off + 12 * V], np.float32).reshape(-1, 3)
    off += 12 * V
    nrm = np.frombuffer(raw[off:off + 12 * V], np.float32).reshape(-1, 3)
    off += 12 * V
    tris = np.frombuffer(raw[off:off + 24 * T], np.uint64).reshape(-1, 3)
    return pts, nrm, tris


@pytest.mark.gpu
def test_shim_meshes_match_oracle(built, cuda, tmp_path):
    import miniisosurface_gb300 as M

    exe = build_shim_check(tmp_path / "shim_check")
    dims, iso = (40, 33, 27), 0.3
    fe_out, mc_out = tmp_path / "fe.bin", tmp_path / "mc.bin"
    run([exe, *dims, iso, fe_out, mc_out])
    vol = M.generate_blobs(dims, 6, seed=21)
    spacing, origin = (0.5, 1.0, 2.0), (-1.0, 0.25, 3.0)
    for path, ref in ((fe_out, oracle_lib.fe(vol, iso, spacing, origin)),
                      (mc_out, oracle_lib.mc(vol, iso, spacing, origin))):
        p, n, t = read_dump(path)
        rp, rn, rt = ref[:3]
        assert len(t) > 0
        assert np.array_equal(t, rt.astype(np.uint64))
        assert np.array_equal(p.view(np.uint32), np.ascontiguousarray(rp).view(np.uint32))
        assert np.array_equal(n.view(np.uint32), np.ascontiguousarray(rn).view(np.uint32))
