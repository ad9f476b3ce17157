"""The screened FP32 assignment's candidate-list guard (times-c_gb300/csrc/
screen.cuh), compiled for the CPU: a list the tensor-core pass did not write
in full makes the FFT pass evaluate every centroid instead of indexing the
centroid spectra with stale values."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_screen_list_guard(tmp_path):
    exe = str(tmp_path / "screen_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "times-c_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "screen_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "ALL OK" in r.stdout
