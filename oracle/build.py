"""Build recipe for the oracle (test infrastructure).

* liboracle.so  - the FP64 restatement (oracle.cpp), g++ -O2 -fopenmp.
* _ref/ref_harness - the reference's own host-side code (its text reader and
  label writer, its random centroid-row draw and its FFT-size rule) compiled
  with nvcc from the reference headers where they lie, plus a small driver of
  ours.  Built only where the reference tree is present; outputs go only to
  oracle/_ref/.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("TIMESC_REFERENCE", "/root/reference")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("command failed: " + " ".join(cmd))
    return r.stdout


def oracle_cmd():
    os.makedirs(BUILD, exist_ok=True)
    return ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
            os.path.join(HERE, "oracle.cpp"), "-o", os.path.join(BUILD, "liboracle.so")]


def build_oracle():
    _run(oracle_cmd())
    return os.path.join(BUILD, "liboracle.so")


def ref_cmd():
    inc = os.path.join(REFERENCE_ROOT, "Code", "include")
    if not os.path.isdir(inc):
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


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
