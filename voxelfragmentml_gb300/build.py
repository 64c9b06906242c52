"""Build libvfgb300.so (the C-ABI library) for sm_103a with nvcc.

Each .cu translation unit compiles in parallel; the objects link into
voxelfragmentml_gb300/_build/libvfgb300.so.  Float code is compiled without
contraction (-fmad=false on the device, -ffp-contract=off on the host) so
that every rounding step matches the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvfgb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["vf_voxelize.cu", "vf_gridops.cu", "vf_flood.cu", "vf_plain.cu",
           "vf_runtime.cu", "vf_api.cu", "vf_noalloc.cu", "vf_rle.cu", "vf_mesh.cu", "vf_impact.cu", "vf_sample.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                   "-prec-sqrt=true", "-ftz=false",
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
                   "-I", INCLUDE, "-I", SRC, *extra]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps += [os.path.join(INCLUDE, "vf.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def one(src):
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *_flags(["-Xptxas", "-v"] if ptxas_v else []), "-c",
               os.path.join(SRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(one, SOURCES))
    if verbose or ptxas_v:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv))
