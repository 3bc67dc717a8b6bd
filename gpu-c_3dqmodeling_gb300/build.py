"""Build libqp3d.so in-tree for sm_103a.

nvcc for the two CUDA translation units (kernels with -fmad=false so that
only the explicitly written fmaf() calls fuse), g++ for the host utilities
(-ffp-contract=off for the same reason), compiled in parallel and linked into
``lib/libqp3d.so`` next to this file.  The CUDA runtime is linked statically;
the driver is reached through cudaGetDriverEntryPointByVersion, so the library
loads on a machine without a GPU driver (its entry points then return
QP3D_ERR_CUDA).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libqp3d.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE]
SOURCES = [
    ("qp3d_kernels.cu", [NVCC] + CU_FLAGS + ["-fmad=false"]),
    ("qp3d_api.cu", [NVCC] + CU_FLAGS),
    ("qp3d_noalloc.cu", [NVCC] + CU_FLAGS),
    ("qp3d_batch.cu", [NVCC] + CU_FLAGS),
    ("qp3d_adjoint.cu", [NVCC] + CU_FLAGS),
    ("qp3d_host.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                       "-Wall", "-I", INCLUDE, "-I", "/usr/local/cuda/include"]),
    ("qp3d_driver.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-Wall", "-I", INCLUDE, "-I", "/usr/local/cuda/include"]),
]
MAIN = ("qp3d_main.cpp", ["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE])
EXE = os.path.join(HERE, "bin", "qp3d_modeling")
HEADERS = ["qp3d_internal.h", "qp3d_exact.h", "qp3d_ctx.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(item, force):
    name, cmd = item
    src = os.path.join(CSRC, name)
    obj = os.path.join(OBJ, name + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    if force or _newer(obj, deps):
        r = subprocess.run(cmd + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (name, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda it: _compile(it, force), SOURCES))
    if force or _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed\n%s\n%s" % (r.stdout, r.stderr))
    # the modeling program, linked against the library next to it
    main_obj = _compile(MAIN, force)
    if force or _newer(EXE, [main_obj, LIB]):
        os.makedirs(os.path.dirname(EXE), exist_ok=True)
        cmd = ["g++", "-o", EXE, main_obj, "-L", os.path.dirname(LIB), "-lqp3d",
               "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link of qp3d_modeling failed\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
