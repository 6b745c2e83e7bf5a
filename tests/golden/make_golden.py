#!/usr/bin/env python3
"""Generate tests/golden/golden.json (+ small .npy volumes) by running the
reference programs built from the miniIsosurface sources by
oracle/build_ref.sh (flyingEdgesSerial, mcSerial).

Each case records the input (a committed .npy volume, or generator
parameters plus the volume's sha256), the isovalue / spacing / origin, and
for each algorithm the vertex and triangle counts and sha256 digests of the
reference's points, normals (little-endian float32) and triangles
(little-endian uint64), and of the reference's output .vtk file.

Usage: python tests/golden/make_golden.py   (needs oracle/_ref/ built)
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))
import oracle_lib  # noqa: E402


def sha(b):
    return hashlib.sha256(b).hexdigest()


def cases():
    import miniisosurface_gb300 as M

    rng = np.random.default_rng(20240601)
    out = []
    # config 0: 128^3 blobs, seed 0, isovalue 0.5 (generator parameters only)
    out.append(dict(name="blobs128_config0", gen=dict(kind="blobs", dims=[128, 128, 128], nblobs=8, seed=0),
                     iso=0.5, spacing=[1, 1, 1], origin=[0, 0, 0],
                     volume=M.generate_blobs((128, 128, 128), 8, seed=0)))
    out.append(dict(name="noise96x80x72", gen=dict(kind="noise", dims=[96, 80, 72], octaves=4, period=64, seed=1),
                     iso=0.0, spacing=[1, 1, 1], origin=[0, 0, 0],
                     volume=M.generate_value_noise((96, 80, 72), 4, 64, seed=1)))
    vol = M.generate_blobs((37, 29, 23), 8, seed=5)
    out.append(dict(name="blobs_spacing", npy="blobs_spacing.npy", iso=0.45, spacing=[0.1, 0.37, 1.3],
                    origin=[-2.5, 0.3, 7.1], volume=vol))
    vol = rng.standard_normal((9, 7, 11)).astype(np.float32)
    out.append(dict(name="gauss_small", npy="gauss_small.npy", iso=0.1, spacing=[1, 1, 1], origin=[0, 0, 0],
                    volume=vol))
    vol = rng.integers(-2, 3, size=(6, 8, 10)).astype(np.float32)
    out.append(dict(name="integer_ties", npy="integer_ties.npy", iso=0.0, spacing=[1, 1, 1], origin=[0, 0, 0],
                    volume=vol))
    vol = rng.standard_normal((5, 4, 2)).astype(np.float32)
    out.append(dict(name="nx2", npy="nx2.npy", iso=0.0, spacing=[0.5, 0.5, 0.5], origin=[1, 1, 1], volume=vol))
    vol = np.ones((4, 4, 4), np.float32)
    out.append(dict(name="all_above", npy="all_above.npy", iso=0.5, spacing=[1, 1, 1], origin=[0, 0, 0],
                    volume=vol))
    return out


def main():
    if not oracle_lib.ref_available("flyingEdgesSerial"):
        sys.exit("reference programs not built: sh oracle/build_ref.sh")
    records = []
    for c in cases():
        vol = c.pop("volume")
        rec = dict(c)
        rec["volume_sha256"] = sha(np.ascontiguousarray(vol, "<f4").tobytes())
        rec["shape_zyx"] = list(vol.shape)
        if "npy" in c:
            np.save(HERE / c["npy"], vol)
        for algo, prog in (("fe", "flyingEdgesSerial"), ("mc", "mcSerial")):
            p, n, t, _, vtk = oracle_lib.run_ref(prog, vol, c["iso"], c["spacing"], c["origin"])
            rec[algo] = dict(n_points=int(p.shape[0]), n_tris=int(t.shape[0]),
                             points=sha(np.ascontiguousarray(p, "<f4").tobytes()),
                             normals=sha(np.ascontiguousarray(n, "<f4").tobytes()),
                             tris=sha(np.ascontiguousarray(t, "<u8").tobytes()),
                             vtk=sha(vtk))
        records.append(rec)
        print(rec["name"], rec["fe"]["n_points"], rec["fe"]["n_tris"])
    (HERE / "golden.json").write_text(json.dumps(records, indent=1) + "\n")


if __name__ == "__main__":
    main()
