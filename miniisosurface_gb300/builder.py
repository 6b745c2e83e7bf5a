"""In-tree build of libminiiso.so (CUDA kernels for sm_103a + C ABI + host IO).

nvcc compiles the .cu translation units and g++ the host .cpp ones, in
parallel; nvcc links the shared library into miniisosurface_gb300/lib/.
Nothing is installed into site-packages.  A build is skipped when the
library is newer than every source.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
OBJDIR = LIBDIR / "obj"
INCLUDE = PKG.parent / "include"
LIBNAME = "libminiiso.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libminiiso")


def library_path():
    return LIBDIR / LIBNAME


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    deps = cu + cpp + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, deps


def _up_to_date(deps):
    lib = library_path()
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(map(str, cmd)), res.stdout, res.stderr))
    return res


def build(verbose=False, force=False):
    """Compile and link libminiiso.so; returns its path."""
    cu, cpp, deps = _sources()
    if not force and _up_to_date(deps):
        return library_path()
    OBJDIR.mkdir(parents=True, exist_ok=True)
    nvcc = nvcc_path()
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    for src in cu:
        obj = OBJDIR / (src.stem + ".cu.o")
        jobs.append(([nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj], obj))
    for src in cpp:
        obj = OBJDIR / (src.stem + ".cpp.o")
        jobs.append(([cxx, *CXX_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj], obj))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda j: _run(j[0], verbose), jobs))
    tmp = LIBDIR / (LIBNAME + ".tmp")
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *[j[1] for j in jobs], "-Xcompiler", "-fopenmp", "-lgomp"], verbose)
    os.replace(tmp, library_path())
    return library_path()


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
