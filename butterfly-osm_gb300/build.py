"""Build recipe for the engine's native libraries (nvcc / g++, no cmake).

Outputs (git-ignored, rebuilt on each machine):
  lib/libbf_phast.so  CUDA engine + C ABI of include/bf_phast.h (sm_103a)
  lib/libbf_cch.so    host CCH build pipeline of cch/bf_cch.h
"""
import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
LIB = PKG / "lib"
OBJ = PKG / "_build"
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_UNITS = ["graph", "engine_plain", "engine_batched", "schedule", "isochrone", "seeded", "twochannel", "customize", "contour", "trace", "tile", "server", "noalloc", "api"]
CU_HEADERS = ["engine.cuh", "scan.cuh"]


def _stale(out, deps):
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(map(str, cmd)), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build_engine(verbose=False):
    """Compile csrc/*.cu for sm_103a and link lib/libbf_phast.so."""
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    csrc = PKG / "csrc"
    headers = [csrc / h for h in CU_HEADERS] + [ROOT / "include" / "bf_phast.h"]
    units = [u for u in CU_UNITS if (csrc / (u + ".cu")).exists()]
    objs = []
    jobs = []
    for u in units:
        src, obj = csrc / (u + ".cu"), OBJ / (u + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-O3", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
                         "-c", str(src), "-o", str(obj)])
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for log in logs:
            print(log)
    so = LIB / "libbf_phast.so"
    if jobs or _stale(so, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(so), *map(str, objs), "-lpthread"])
    return so


def build_cch():
    """Compile cch/cch_build.cpp into lib/libbf_cch.so."""
    LIB.mkdir(exist_ok=True)
    src = PKG / "cch" / "cch_build.cpp"
    so = LIB / "libbf_cch.so"
    if _stale(so, [src, PKG / "cch" / "bf_cch.h"]):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
              str(src), "-o", str(so)])
    return so


def build_all(verbose=False):
    with concurrent.futures.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_engine, verbose)
        b = ex.submit(build_cch)
        return a.result(), b.result()


if __name__ == "__main__":
    print(build_all(verbose=True))
