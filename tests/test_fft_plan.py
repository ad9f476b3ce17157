"""CPU emulation of the fused SBD transform plan (no GPU): the per-thread
phases of times-c_gb300/csrc/sbd_core.cuh run for every supported transform
size and are compared with direct FP64 correlation sums."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sbd_core_plan_all_sizes(tmp_path):
    exe = str(tmp_path / "sbd_core_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", "/usr/local/cuda/include",
                    "-I", os.path.join(ROOT, "times-c_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "sbd_core_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "ALL OK" in r.stdout
