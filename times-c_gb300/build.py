"""Build recipe of the engine: libtimesc.so (CUDA kernels + C ABI) and the
`test` CLI, compiled in-tree for sm_103a with nvcc/g++ (no cmake).

Objects go to times-c_gb300/_build/, the library to times-c_gb300/lib/, the
CLI to times-c_gb300/bin/.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
BIN_DIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIB_DIR, "libtimesc.so")
CLI = os.path.join(BIN_DIR, "test")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
             "-I", "/usr/local/cuda/include"]

CU_SOURCES = ["assign_fft.cu", "znorm.cu", "extract.cu", "power.cu", "power_sq.cu", "tensor_core.cu", "assign_tc.cu",
              "loop_graph.cu"]
CPP_SOURCES = ["api.cpp", "io.cpp", "gen.cpp", "pool.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout)
        raise RuntimeError("build step failed: " + os.path.basename(cmd[-1]))
    return r.stdout


def _obj(src):
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def _needs(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "timesc.h")]


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    hdr = _headers()
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        if _needs(_obj(s), [src] + hdr):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append(["nvcc"] + NVCC_FLAGS + extra + ["-c", src, "-o", _obj(s)])
    for s in CPP_SOURCES + ["cli.cpp"]:
        src = os.path.join(CSRC, s)
        if _needs(_obj(s), [src] + hdr):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", _obj(s)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [_obj(s) for s in CU_SOURCES + CPP_SOURCES]
    if _needs(LIB, objs):
        _run(["nvcc"] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"])
    if _needs(CLI, [_obj("cli.cpp"), LIB]):
        _run(["g++", "-o", CLI, _obj("cli.cpp"), "-L", LIB_DIR, "-ltimesc", "-Wl,-rpath,$ORIGIN/../lib",
              "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
