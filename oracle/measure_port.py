#!/usr/bin/env python3
"""Times the oracle port against the reference's own CPU programs on one host.

The GPU host has no reference checkout and no compiler for the reference's
programs can reach it from here, so the CPU arm there times the oracle
port (oracle/fe_oracle.c, oracle/mc_oracle.c).  This script measures, on the
host where oracle/build_ref.sh built the programs, how the port's extraction
time compares with each program's own "Total Program WALL Time" on the same
volume, so that the port's numbers can be read as the reference's:

    flyingEdgesSerial  vs  oracle_fe_run, 1 thread
    flyingEdgesOpenMP  vs  oracle_fe_run, all threads
    mcSerial           vs  oracle_mc_run
    mcOpenMP           vs  oracle_mc_openmp_run, all threads

Best of --reps runs each.  Writes oracle/port_factors.json (factor =
program seconds / port seconds; above 1 means the port is faster).

Usage: python oracle/measure_port.py [--dims 512] [--reps 3]
"""
import argparse
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent / "tests"))
import oracle_lib  # noqa: E402

LEGS = (("flyingEdgesSerial", "fe", 1), ("flyingEdgesOpenMP", "fe", 0), ("mcSerial", "mc", 1),
        ("mcOpenMP", "mc_openmp", 0))


def cpu_model():
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def program_seconds(prog, vin, threads, reps):
    best = None
    with tempfile.TemporaryDirectory() as td:
        for _ in range(reps):
            ym = os.path.join(td, "run.yaml")
            subprocess.run([str(oracle_lib.REF_DIR / prog), "-i", vin, "-o", os.path.join(td, "out.vtk"), "-v", "0.0",
                            "-y", ym], env=dict(os.environ, OMP_NUM_THREADS=str(threads)), capture_output=True,
                           check=True)
            m = re.search(r"Total Program WALL Time \(seconds\):\s*([0-9.eE+-]+)", Path(ym).read_text())
            t = float(m.group(1))
            best = t if best is None else min(best, t)
    return best


def port_seconds(kind, vol, threads, reps):
    best = None
    for _ in range(reps):
        if kind == "fe":
            oracle_lib.fe(vol, 0.0, nthreads=threads)
            t = oracle_lib.fe_wall_seconds()
        elif kind == "mc":
            oracle_lib.mc(vol, 0.0)
            t = oracle_lib.mc_wall_seconds()
        else:
            oracle_lib.mc_openmp(vol, 0.0, nthreads=threads)
            t = oracle_lib.mc_wall_seconds()
        best = t if best is None else min(best, t)
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, default=512)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    if not oracle_lib.ref_available("flyingEdgesOpenMP"):
        sys.exit("reference programs not built: sh oracle/build_ref.sh")
    n = args.dims
    vol = oracle_lib.generate_value_noise((n, n, n), 4, 64, 1)
    cores = os.cpu_count() or 1
    out = {"host": {"arch": platform.machine(), "cpu": cpu_model(), "cores": cores},
           "volume": "%d^3 float32, 4-octave value noise, base period 64, seed 1, isovalue 0" % n,
           "reps": args.reps, "legs": {}}
    with tempfile.TemporaryDirectory() as td:
        vin = os.path.join(td, "in.vtk")
        oracle_lib.write_structured_points(vin, vol)
        for prog, kind, thr in LEGS:
            threads = thr or cores
            tp = program_seconds(prog, vin, threads, args.reps)
            to = port_seconds(kind, vol, threads, args.reps)
            out["legs"][prog] = {"threads": threads, "program_s": tp, "port_s": to, "factor": tp / to}
            print("%-18s %2d threads  program %.3f s  port %.3f s  factor %.3f" % (prog, threads, tp, to, tp / to),
                  flush=True)
    (HERE / "port_factors.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
