"""Build the native libraries in-tree (``vnec_gb300/_lib``).

* ``libvnec_gb300.so`` — the C-ABI library: CUDA kernels compiled for sm_103a
  only, host plan code compiled with OpenMP.
* ``libvnec_gen.so`` — seeded synthetic matrix generators (host only).

Translation units are compiled in parallel and only when a source or header
is newer than its object, so repeated builds are quick.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "_lib")
OBJ = os.path.join(LIB, "obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}")


def build(verbose: bool = False, ptxas_info: bool = False) -> dict[str, str]:
    os.makedirs(OBJ, exist_ok=True)
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    headers = (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
               glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(p for p in glob.glob(os.path.join(CSRC, "*.cpp")) if not p.endswith("generators.cpp"))
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
                   "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in cpp:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-I", INCLUDE, "-I", CSRC,
                         "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj])
    gen_src = os.path.join(CSRC, "generators.cpp")
    gen_lib = os.path.join(LIB, "libvnec_gen.so")
    if _newer(gen_lib, [gen_src]):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-shared", gen_src, "-o", gen_lib])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, jobs))
    lib = os.path.join(LIB, "libvnec_gb300.so")
    if _newer(lib, objs):
        libdirs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                               os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                               os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(d)]
        cmd = ["g++", "-shared", "-fopenmp", "-o", lib, *objs]
        for d in libdirs:
            cmd += ["-L", d, f"-Wl,-rpath,{d}"]
        cmd += ["-lcudart", "-lgomp"]
        _run(cmd)
    return {"vnec_gb300": lib, "vnec_gen": gen_lib}


if __name__ == "__main__":
    out = build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    for k, v in out.items():
        print(k, v)
