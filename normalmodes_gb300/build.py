"""Build recipe for the native libraries of the package.

Everything is compiled in-tree with plain compiler invocations (no cmake):

* ``libnmmodel.so`` -- host C++ (g++ -fopenmp): synthetic models and FEM
  assembly (the input side of the eigensolve path).
* ``libnmgpu.so``   -- CUDA for sm_103a (nvcc): the GPU eigensolver behind the
  C-ABI declared in ``include/nmgpu.h``.

The oracle under ``oracle/`` has its own recipe (``oracle.build()`` in
``oracle/oracle.py``) because it is test infrastructure, not part of the
product.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIBDIR = os.path.join(PKG, "lib")
CSRC = os.path.join(PKG, "csrc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

MODEL_SRC = [os.path.join(CSRC, "model", "nm_model.cpp")]
GPU_CU = sorted(
    os.path.join(CSRC, "gpu", f)
    for f in os.listdir(os.path.join(CSRC, "gpu"))
    if f.endswith(".cu")
) if os.path.isdir(os.path.join(CSRC, "gpu")) else []
GPU_CPP = sorted(
    os.path.join(CSRC, "gpu", f)
    for f in os.listdir(os.path.join(CSRC, "gpu"))
    if f.endswith(".cpp")
) if os.path.isdir(os.path.join(CSRC, "gpu")) else []


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {os.path.basename(cmd[-1])}")


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = list(srcs)
    for d in (os.path.join(ROOT, "include"), os.path.join(CSRC, "gpu"), os.path.join(CSRC, "model")):
        if os.path.isdir(d):
            deps += [os.path.join(d, f) for f in os.listdir(d)]
    return any(os.path.getmtime(s) > t for s in deps if os.path.isfile(s))


def build_model(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libnmmodel.so")
    if force or _stale(out, MODEL_SRC):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-unused-function",
              "-o", out] + MODEL_SRC)
    return out


def build_gpu(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libnmgpu.so")
    srcs = GPU_CU + GPU_CPP
    if not srcs:
        raise RuntimeError("no GPU sources")
    if not (force or _stale(out, srcs)):
        return out
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for s in GPU_CU:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                               "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                               "-c", s, "-o", o]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append(cmd)
    for s in GPU_CPP:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall",
                     "-I", os.path.join(ROOT, "include"),
                     "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
                     "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", out] + objs +
         ["-lcudart", "-lcublas", "-lcusolver", "-lgomp"])
    return out


def build_all(force: bool = False) -> list[str]:
    outs = [build_model(force)]
    if GPU_CU:
        outs.append(build_gpu(force))
    return outs


if __name__ == "__main__":
    for p in build_all(force="--force" in sys.argv):
        print(p)
