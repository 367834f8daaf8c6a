"""Builds the native parts in-tree:
  libexastitch.so -- the CUDA path (sm_103a kernels + C++ host + C ABI)
  libexagen.so    -- the dataset generator (host C++ and its CUDA version)
Compiles translation units in parallel and skips up-to-date outputs.

    python -m owlexastitcher_gb300.build
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no contracted multiply-add, so float results follow the
# source's operation order exactly (the CPU oracle builds the same way)
NVFLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-I" + INCLUDE, "-I" + CSRC]
CUDA_SOURCES = ["exa_build.cu", "exa_render.cu", "exa_surrogate.cu", "exa_exabrick.cu", "exa_api.cpp"]
HEADERS = ["exa_device.cuh", "exa_accel.cuh", "exa_host.h", "exa_mesh.cuh", "exa_surrogate.cuh", "exa_tcgen05.cuh"]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True, stdin=subprocess.DEVNULL)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_exastitch(verbose=False, variant=None):
    """variant "checks": libexastitch_checks.so, built with EXA_CHECKS=1 (the
    kernels test every index they read through before the access, record
    EXA_DEVERR_BOUNDS and skip it), objects in _build/checks"""
    build = BUILD if variant is None else os.path.join(BUILD, variant)
    os.makedirs(build, exist_ok=True)
    out = os.path.join(PKG, "libexastitch.so" if variant is None else f"libexastitch_{variant}.so")
    vflags = [] if variant is None else {"checks": ["-DEXA_CHECKS=1"]}[variant]
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "exastitch.h")]
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build, src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            # EXA_NVCC_EXTRA: extra nvcc flags (e.g. -DEXA_RENDER_MIN_BLOCKS=3)
            extra = os.environ.get("EXA_NVCC_EXTRA", "").split()
            cmd = [nvcc()] + ARCH + NVFLAGS + vflags + extra + ["-x", "cu", "-c", s, "-o", o]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for log in ex.map(_run, jobs):
            if verbose and log:
                print(log)
    if _newer(out, objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", out] + objs)
    return out


def build_exagen():
    """libexagen.so: the CPU generator (g++, OpenMP) and its GPU version
    (nvcc), both without contracted multiply-adds so that they evaluate the
    shared field code identically."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(PKG, "libexagen.so")
    gen = os.path.join(CSRC, "gen")
    hdrs = [os.path.join(gen, h) for h in ("exagen_field.h", "exagen_internal.h")] + [
        os.path.join(INCLUDE, "exastitch_gen.h"), os.path.join(INCLUDE, "exastitch.h")]
    cpu_src, gpu_src = os.path.join(gen, "exagen.cpp"), os.path.join(gen, "exagen_gpu.cu")
    cpu_obj, gpu_obj = os.path.join(BUILD, "exagen.cpp.o"), os.path.join(BUILD, "exagen_gpu.cu.o")
    jobs = []
    if _newer(cpu_obj, [cpu_src] + hdrs):
        cxx = shutil.which("g++") or "g++"
        jobs.append([cxx, "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-Wall", "-c", cpu_src,
                     "-o", cpu_obj])
    if _newer(gpu_obj, [gpu_src] + hdrs):
        jobs.append([nvcc()] + ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                                       "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off",
                                       "-Xcompiler", "-Wall", "-c", gpu_src, "-o", gpu_obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if _newer(out, [cpu_obj, gpu_obj]):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-Xcompiler", "-fopenmp", "-o", out, cpu_obj,
                                gpu_obj, "-lgomp"])
    return out


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_exastitch, verbose)
        b = ex.submit(build_exagen)
        return a.result(), b.result()


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
