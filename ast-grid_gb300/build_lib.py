"""Builds libastgrid_gpu.so in-tree (ast-grid_gb300/_build/) with nvcc for sm_103a.

FMA contraction is off in device and host code so the FP64 step follows the reference's IEEE
operation order; where the kernels fuse a multiply and an add they say so with an explicit fma().
The FP32 kernels of the mixed form are built under the same flag; their sweeps are bound by the
dependency chain (latency), not by arithmetic, so contraction would not change their speed much."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libastgrid_gpu.so")
SOURCES = ["astg_host.cpp", "astg_step.cu", "astg_pcg.cu", "astg_extrap.cu", "astg_adjoint.cu", "astg_collider.cu",
           "astg_layout.cu",
           "astg2d.cu", "astg2d_host.cpp"]
HEADERS = ["astg_device.cuh", "astg_sample.cuh", "astg_launch.h", "astg2d_launch.h", "scene.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", h) for h in ("astg.h", "astg2d.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [sp] + hdrs):
            jobs.append([_nvcc()] + FLAGS + ARCH + ["-c", sp, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([_nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    return LIB


EXAMPLE_SRC = os.path.join(HERE, "examples", "octree_smoke.cpp")
EXAMPLE = os.path.join(BUILD, "octree_smoke")


def build_example(force=False):
    """examples/octree_smoke.cpp, a C++ program using only include/astg.h, linked against the
    library (found next to it at run time)."""
    lib = build(force=force)
    if force or _stale(EXAMPLE, [EXAMPLE_SRC, lib, os.path.join(ROOT, "include", "astg.h")]):
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), EXAMPLE_SRC, "-o",
               EXAMPLE + ".tmp", "-L", BUILD, "-lastgrid_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("example build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(EXAMPLE + ".tmp", EXAMPLE)
    return EXAMPLE


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_example())
