"""Build recipe for the oracle (test infrastructure).

* liboracle.so  - the FP64 restatement (oracle.cpp), g++ -O2 -fopenmp, plus the
  engine's synthetic-workload generator (the header times-c_gb300/csrc/gen_core.h)
  so that the CPU baseline makes the same series without the engine's library.
* _ref/ref_harness - the reference's own host-side code (its text reader and
  label writer, its random centroid-row draw and its FFT-size rule) compiled
  with nvcc from the reference headers where they lie, plus a small driver of
  ours.  Built only where the reference tree is present; outputs go only to
  oracle/_ref/.
* _ref/src/include - a staged, git-ignored copy of the reference's headers
  (Code/include/*.cuh), made where the reference tree is present.  The GPU host
  has no reference tree; the copy travels with the working tree.
* _ref/ref_gpu - the reference's GPU code (its z-norm, NCC_3D + get_pos_idx,
  extract_shape and k_shape / k_shape_tsl loops, linked with cuBLAS, cuFFT,
  cuSOLVER and cuRAND as its Makefile does) around our driver
  ref_gpu_harness.cu, compiled on the GPU host from the staged copy for
  sm_103a.  No reference file is edited: the seeded random_device shim is
  force-included, and the one line of the reference's CLI that no longer
  compiles with CUDA 13 (clockRate, Code/test/test_kshape.cu:186) is in the
  part of the CLI our driver replaces.

The reference tree is TIMESC_REFERENCE, else the directory `reference` beside
the repository.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(REF_OUT, "src", "include")
REF_GPU = os.path.join(REF_OUT, "ref_gpu")
REFERENCE_ROOT = os.environ.get("TIMESC_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("command failed: " + " ".join(cmd))
    return r.stdout


def oracle_cmd():
    os.makedirs(BUILD, exist_ok=True)
    return ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
            "-I", os.path.join(ROOT, "times-c_gb300", "csrc"),
            os.path.join(HERE, "oracle.cpp"), "-o", os.path.join(BUILD, "liboracle.so")]


def build_oracle():
    _run(oracle_cmd())
    return os.path.join(BUILD, "liboracle.so")


def reference_include():
    inc = os.path.join(REFERENCE_ROOT, "Code", "include")
    return inc if os.path.isdir(inc) else None


def ref_cmd():
    inc = reference_include()
    if inc is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    return ["nvcc", "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
            "-include", os.path.join(HERE, "ref_shim.h"), "-I", inc,
            os.path.join(HERE, "ref_harness.cu"), "-o", os.path.join(REF_OUT, "ref_harness"),
            "-lcublas", "-lcufft", "-lcusolver", "-lcurand"]


def build_ref():
    cmd = ref_cmd()
    if cmd is None:
        return None
    _run(cmd)
    return os.path.join(REF_OUT, "ref_harness")


def stage_ref_gpu():
    """Copies the reference headers to oracle/_ref/src/include (git-ignored).
    Returns the staged directory, or None where the reference tree is absent."""
    inc = reference_include()
    if inc is None:
        return REF_SRC if os.path.isdir(REF_SRC) else None
    os.makedirs(REF_SRC, exist_ok=True)
    for name in sorted(os.listdir(inc)):
        if name.endswith((".cuh", ".h")):
            src, dst = os.path.join(inc, name), os.path.join(REF_SRC, name)
            if not os.path.exists(dst) or open(src, "rb").read() != open(dst, "rb").read():
                shutil.copyfile(src, dst)
    return REF_SRC


def ref_gpu_cmd():
    if not os.path.isdir(REF_SRC):
        return None
    # The reference's Makefile: -rdc=true, cuBLAS, cuFFT, cuSOLVER, cuRAND
    # (Code/Makefile:17-25), here for sm_103a.
    return ["nvcc", "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true",
            "-include", os.path.join(HERE, "ref_shim.h"), "-I", REF_SRC,
            os.path.join(HERE, "ref_gpu_harness.cu"), "-o", REF_GPU,
            "-lcublas", "-lcufft", "-lcusolver", "-lcurand", "-lcudadevrt"]


def build_ref_gpu():
    """Compiles oracle/_ref/ref_gpu from the staged headers (on the GPU host,
    where binaries built elsewhere do not run).  Returns its path or None."""
    stage_ref_gpu()
    cmd = ref_gpu_cmd()
    if cmd is None:
        return None
    deps = [os.path.join(HERE, "ref_gpu_harness.cu"), os.path.join(HERE, "ref_shim.h")] + \
        [os.path.join(REF_SRC, f) for f in os.listdir(REF_SRC)]
    if os.path.exists(REF_GPU) and all(os.path.getmtime(d) <= os.path.getmtime(REF_GPU) for d in deps):
        return REF_GPU
    _run(cmd)
    return REF_GPU


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(stage_ref_gpu())
    if len(sys.argv) > 1 and sys.argv[1] == "ref_gpu":
        print(build_ref_gpu())
