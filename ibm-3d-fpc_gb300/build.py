"""Build recipe of the package's native libraries (in-tree, under _build/).

libibmhost.so : CPU setup (csrc/host), g++ -O2 -ffp-contract=off.
libibmgpu.so  : the CUDA solver (csrc/cuda), nvcc for sm_103a only.

Translation units compile in parallel; objects are rebuilt when a source or
header is newer. Run as ``python build.py`` from this directory or call
:func:`build_all`.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + os.path.join(HERE, "csrc", "cuda")] + GENCODE


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd[:6]) + " ...")


def build_host() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "csrc", "host", "ibm_setup.cpp")
    out = os.path.join(BUILD, "libibmhost.so")
    deps = [src, os.path.join(INCLUDE, "ibm_host.h")]
    if _newer(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-I" + INCLUDE,
              src, "-o", out])
    return out


def build_gpu(jobs: int = 8) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(HERE, "csrc", "cuda", "*.cu")))
    hdrs = glob.glob(os.path.join(HERE, "csrc", "cuda", "*.cuh")) + [os.path.join(INCLUDE, "ibm_gpu.h")]
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            todo.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for f in [ex.submit(_run, c) for c in todo]:
            f.result()
    out = os.path.join(BUILD, "libibmgpu.so")
    if _newer(out, objs):
        _run([NVCC] + GENCODE + ["-shared", "-o", out] + objs + ["-lcudart"])
    return out


def build_driver() -> str:
    """ibm_run: the reference's application (main.cu) on the two C ABIs."""
    src = os.path.join(HERE, "csrc", "driver", "ibm_run.cpp")
    out = os.path.join(BUILD, "ibm_run")
    deps = [src, os.path.join(INCLUDE, "ibm_gpu.h"), os.path.join(INCLUDE, "ibm_host.h"),
            os.path.join(BUILD, "libibmgpu.so"), os.path.join(BUILD, "libibmhost.so")]
    if _newer(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, src, "-o", out, "-L" + BUILD, "-libmgpu",
              "-libmhost", "-Wl,-rpath,$ORIGIN"])
    return out


def build_all() -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fs = [ex.submit(build_host), ex.submit(build_gpu)]
        for f in fs:
            f.result()
    build_driver()


if __name__ == "__main__":
    build_all()
    print("built", os.listdir(BUILD))
