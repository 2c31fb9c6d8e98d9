"""Build of liblgca_gpu.so: nvcc for sm_103a, one object per CUDA source,
compiled in parallel, linked in-tree as lgca_gb300/liblgca_gpu.so."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblgca_gpu.so")
SOURCES = ["step.cu", "multistep.cu", "wave.cu", "aux.cu", "bodyforce.cu", "batch.cu",
           "lgca_gpu.cu", "noalloc.cu", "resident.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
APPS = {"lgca_headless": "apps/lgca_headless.cpp"}
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblgca_gpu.so")


def app_path(name: str) -> str:
    return os.path.join(BUILD, name)


def _deps() -> list[str]:
    inc = os.path.join(os.path.dirname(PKG), "include")
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    for root, _, names in os.walk(inc):
        files += [os.path.join(root, n) for n in names]
    return files


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source of the package and link liblgca_gpu.so."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in srcs]

    def compile_one(src, obj):
        if not force and not _stale(obj, deps):
            return
        cmd = [cc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        list(ex.map(lambda so: compile_one(*so), zip(srcs, objs)))
    if force or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    # headless application drivers (host C++ over the C ABI)
    inc = os.path.join(os.path.dirname(PKG), "include")
    for name, src in APPS.items():
        out = app_path(name)
        src = os.path.join(PKG, src)
        if force or _stale(out, deps + [src, LIB]):
            cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I", inc, src, "-o", out,
                   "-L", PKG, "-llgca_gpu", "-Wl,-rpath,$ORIGIN/.."]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"g++ failed on {src}:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
