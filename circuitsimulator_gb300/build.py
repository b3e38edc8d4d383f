"""Builds the native parts in-tree:

* circuitsimulator_gb300/libcsimgpu.so — CUDA kernels (sm_103a only) + the C ABI
  of include/csim.h;
* circuitsimulator_gb300/gpubackend — the stdin-protocol backend executable;

Usage: ``python -m circuitsimulator_gb300.build`` (or ``build()``).  Uses nvcc
and gcc directly; translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcsimgpu.so")
EXE = os.path.join(PKG, "gpubackend")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps every double rounding explicit (no fused multiply-add
# contraction, which gcc does by default on aarch64), so the estimators give
# the same bits on x86 and Arm hosts and in every code path.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                  "-I" + os.path.join(ROOT, "include")]
SOURCES = ["csim_kernels.cu", "csim_terms_tp.cu", "csim_static.cu", "csim_batch_kernels.cu", "csim_host.cpp",
           "csim_engine.cpp", "csim_backend.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "csim.h"))
    objs, procs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            cmd = [nvcc] + NVFLAGS + ["-c", s, "-o", o]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"] if verbose else []
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), out))
        if verbose and out:
            print(out)
    if force or procs or _newer(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        subprocess.check_call(cmd)
    gb = os.path.join(CSRC, "gpubackend.c")
    if force or _newer(EXE, [gb, LIB]):
        cc = shutil.which("gcc") or "cc"
        subprocess.check_call([cc, "-O2", "-std=gnu99", "-I" + os.path.join(ROOT, "include"), gb, "-o", EXE,
                               "-L" + PKG, "-lcsimgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
