"""In-tree build of the native libraries (no cmake, no setup.py).

  eqdyna_gb300/lib/libeqd_case.so     host case setup (g++)
  eqdyna_gb300/lib/libeqdyna_gb300.so GB300 hot path + C ABI (nvcc, sm_103a only; host setup
                                      loops in OpenMP)
  oracle/liboracle.so                 CPU binary64 restatement used only by tests and the CPU
                                      baseline (g++ -fopenmp)

Every library is rebuilt when one of its sources is newer than the library.  Translation units
are compiled in parallel.  Host code uses -ffp-contract=off so that x86_64 and aarch64 round the
same way.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I" + INCLUDE]
CU_SOURCES = ["eqd_api.cu", "kernels_elem.cu", "kernels_elem32.cu", "kernels_elem32r.cu",
              "kernels_fault.cu", "kernels_mlp.cu", "noalloc.cu", "setup_device.cu"]
# per-file flags: the device table build restates host arithmetic bit for bit, so nothing in it
# may be contracted into a fused multiply-add
CU_FLAGS = {"setup_device.cu": ["--fmad=false"]}
# every header of csrc/ is a dependency of every CUDA translation unit, so that a change to any of
# them (the Newton loop, the conversions, ...) rebuilds the objects that include it
CU_HEADERS = sorted(f for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))

CASE_LIB = os.path.join(LIBDIR, "libeqd_case.so")
GPU_LIB = os.path.join(LIBDIR, "libeqdyna_gb300.so")
ORACLE_LIB = os.path.join(ORACLE, "liboracle.so")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_case(force=False):
    src = os.path.join(CSRC, "case_builder.cpp")
    deps = [src, os.path.join(INCLUDE, "eqdyna_case.h"), os.path.join(INCLUDE, "eqdyna_gb300.h"),
            os.path.join(CSRC, "eqd_geometry.h")]
    if force or _newer(CASE_LIB, deps):
        os.makedirs(LIBDIR, exist_ok=True)
        _run(["g++", *HOST_FLAGS, "-fopenmp", "-shared", src, "-o", CASE_LIB])
    return CASE_LIB


def build_oracle(force=False):
    src = os.path.join(ORACLE, "eqd_oracle.cpp")
    deps = [src, os.path.join(INCLUDE, "eqdyna_gb300.h")]
    if force or _newer(ORACLE_LIB, deps):
        _run(["g++", *HOST_FLAGS, "-fopenmp", "-shared", src, "-o", ORACLE_LIB])
    return ORACLE_LIB


def build_gpu(force=False, verbose_ptxas=False, jobs=None):
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at " + NVCC)
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in CU_HEADERS] + [os.path.join(INCLUDE, "eqdyna_gb300.h")]
    objs, todo = [], []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(LIBDIR, "obj", s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC,
                   *CU_FLAGS.get(s, []), "-c", src, "-o", obj]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            todo.append(cmd)
    out = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            out = list(ex.map(_run, todo))
    if force or todo or _newer(GPU_LIB, objs):
        _run([NVCC, *ARCH, "-shared", *objs, "-o", GPU_LIB, "-lcudart", "-lgomp"])
    return GPU_LIB, "".join(out)


def build_all(force=False, with_oracle=True):
    libs = [build_case(force)]
    if with_oracle:
        libs.append(build_oracle(force))
    libs.append(build_gpu(force)[0])
    return libs


if __name__ == "__main__":
    force = "--force" in sys.argv
    if "--ptxas" in sys.argv:
        print(build_gpu(force=True, verbose_ptxas=True)[1])
    else:
        for lib in build_all(force):
            print(lib)
