"""CPU: the bench's workload generators and link arithmetic."""
import numpy as np

import bench


def test_link_floor_takes_the_binding_limit():
    r = bench.link_floor((200e9, 100e9, 250e9), 400e6, 100e6, 4.0)
    assert abs(r["floor_ms_per_step"] - 2.0) < 1e-9  # host->device bound: 400 MB at 200 GB/s
    assert abs(r["frac_of_floor"] - 0.5) < 1e-9
    r = bench.link_floor((200e9, 100e9, 250e9), 300e6, 300e6, 6.0)
    assert abs(r["floor_ms_per_step"] - 3.0) < 1e-9  # device->host bound: 300 MB at 100 GB/s
    r = bench.link_floor((200e9, 200e9, 250e9), 300e6, 300e6, 6.0)
    assert abs(r["floor_ms_per_step"] - 2.4) < 1e-9  # both directions at once: 600 MB at 250 GB/s


def test_batch_workload_distribution():
    import miniisosurface_gb300 as M
    vols, reqs = bench.batch_workload(M, seed=2, nvol=8)
    assert len(vols) == 8
    per_volume = np.bincount([v for v, _ in reqs], minlength=8)
    assert per_volume.min() >= 1 and per_volume.max() <= 4
    for v, (dims, vol) in enumerate(vols):
        assert all(32 <= d <= 320 for d in dims)
        assert vol.shape == (dims[2], dims[1], dims[0]) and vol.dtype == np.float32
        lo, hi = np.percentile(vol[:: max(1, vol.shape[0] // 16)], [5, 95])
        for vi, iso in reqs:
            if vi == v:
                assert lo - 1e-6 <= iso <= hi + 1e-6
    again = bench.batch_workload(M, seed=2, nvol=8)[1]
    assert again == reqs  # seeded


def test_reference_arm_runs_without_the_product_library(tmp_path):
    """bench.py --impl reference on a small volume, in a fresh process: it
    prints its JSON line with the four CPU legs, and neither the product
    package nor libminiiso.so is ever loaded."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '2', '--warmup', '1'];"
        "import bench; bench.DIMS = (40, 36, 30); bench.main();"
        "maps = open('/proc/self/maps').read();"
        "bad = [m for m in sys.modules if m.startswith('miniisosurface_gb300')];"
        "assert not bad and 'libminiiso' not in maps, (bad, 'libminiiso' in maps)")
    res = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads([x for x in res.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    legs = line["cpu_baseline"]["legs"]
    assert set(legs) == {"flyingEdgesSerial", "flyingEdgesOpenMP", "mcSerial", "mcOpenMP"}
    assert all(v["value"] > 0 and v["kind"] in ("reference", "port") for v in legs.values())
    assert line["e2e"]["h2d_bytes_per_step"] == 0
