"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/lib/libqp3d_oracle.so`` -- the C restatement in qp3d_oracle.c
  (FP32 reference arithmetic, FP64, and the kernel-arithmetic mirror).
* ``oracle/_ref/libqp3d_ref.so`` -- the reference's own CPU_function.c compiled
  in place from the reference checkout plus ref_harness.cpp.
* ``oracle/_ref/gpu_kernel.cubin`` -- the reference's own GPU_kernel.cu,
  unmodified, compiled for sm_103a with nvcc's defaults (as its build script
  compiles it, compile_GPU.sh:8); device code only, so the same file serves
  any host.
* ``oracle/lib/libqp3d_refgpu.so`` -- ref_gpu.cu, the host driver that loads
  that cubin and runs the reference GPU driver's step sequence.

The two ``_ref`` outputs are built only where the reference checkout exists;
its location comes from the command line (``--reference DIR``), else from
QP3D_REFERENCE_DIR, else the checkout location of the build container.
Nothing is copied out of the checkout; the output directories are git-ignored
(and travel with the working tree to a GPU machine, where the cubin is used
as it is and the host-side libraries are rebuilt).

Both are built with ``-ffp-contract=off`` so that no compiler fuses a*b+c and
the FP32 roundings are the ones written in the source, on x86 and on Arm.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "libqp3d_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libqp3d_ref.so")
REF_CUBIN = os.path.join(HERE, "_ref", "gpu_kernel.cubin")
REFGPU_LIB = os.path.join(HERE, "lib", "libqp3d_refgpu.so")
REFERENCE_DIR = os.environ.get("QP3D_REFERENCE_DIR", "/root/reference")
NVCC = os.environ.get("NVCC", "nvcc")

COMMON = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp"]


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "qp3d_oracle.c"), os.path.join(HERE, "qp3d_adjoint.c")]
    hdr = os.path.join(HERE, "qp3d_oracle.h")
    if force or _newer(LIB, srcs + [hdr]):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        cmd = ["gcc", "-std=c11", "-Wall"] + COMMON + ["-o", LIB] + srcs + ["-lm"]
        subprocess.check_call(cmd)
    return LIB


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_DIR, "CPU_function.c"))


def build_reference(force=False):
    """Compile the reference CPU operators; returns the .so path or None."""
    if not reference_available():
        return None
    ref_src = os.path.join(REFERENCE_DIR, "CPU_function.c")
    harness = os.path.join(HERE, "ref_harness.cpp")
    if force or _newer(REF_LIB, [ref_src, harness]):
        os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
        # The reference builds its .c files with g++ (Makefile:9), i.e. as C++.
        cmd = (["g++", "-x", "c++", "-w"] + COMMON +
               ["-Dexchange=qp3d_ref_exchange_unused", "-I", REFERENCE_DIR,
                "-o", REF_LIB, ref_src, harness, "-lm"])
        subprocess.check_call(cmd)
    return REF_LIB


def build_reference_gpu(force=False):
    """Compile the reference GPU kernels into a cubin (checkout needed) and
    the host driver that runs them (always).  Returns (cubin or None, lib)."""
    cubin = None
    if reference_available():
        src = os.path.join(REFERENCE_DIR, "GPU_kernel.cu")
        if force or _newer(REF_CUBIN, [src]):
            os.makedirs(os.path.dirname(REF_CUBIN), exist_ok=True)
            subprocess.check_call([NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                                   "-w", "-I", REFERENCE_DIR, "-o", REF_CUBIN, src])
    if os.path.exists(REF_CUBIN):
        cubin = REF_CUBIN
    drv = os.path.join(HERE, "ref_gpu.cu")
    if force or _newer(REFGPU_LIB, [drv, os.path.join(HERE, "qp3d_oracle.h")]):
        os.makedirs(os.path.dirname(REFGPU_LIB), exist_ok=True)
        subprocess.check_call([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                               "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-o", REFGPU_LIB,
                               drv])
    return cubin, REFGPU_LIB


def build(force=False):
    build_oracle(force)
    build_reference(force)
    build_reference_gpu(force)


if __name__ == "__main__":
    if "--reference" in sys.argv:
        REFERENCE_DIR = sys.argv[sys.argv.index("--reference") + 1]
    build(force="--force" in sys.argv)
    print(LIB)
    print(REF_LIB if os.path.exists(REF_LIB) else "(reference CPU operators not built)")
    print(REF_CUBIN if os.path.exists(REF_CUBIN) else "(reference GPU kernels not built)")
