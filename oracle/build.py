"""Build recipe for the CPU oracle (test infrastructure only).

Compiles phast_oracle.cpp, contour_oracle.cpp and tile_oracle.cpp into
oracle/_build/liboracle.so (no floating-point contraction, so every step
rounds as written). Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg load it.
"""
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build"


def build_oracle():
    OUT.mkdir(exist_ok=True)
    srcs = [HERE / "phast_oracle.cpp", HERE / "contour_oracle.cpp", HERE / "tile_oracle.cpp"]
    so = OUT / "liboracle.so"
    if not so.exists() or any(so.stat().st_mtime < s.stat().st_mtime for s in srcs):
        r = subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                            "-ffp-contract=off", *map(str, srcs), "-o", str(so)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return so


if __name__ == "__main__":
    print(build_oracle())
