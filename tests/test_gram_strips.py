"""The tensor-core Gram's strips (times-c_gb300/csrc/gram_strips.h) compiled for
the CPU: every upper-triangle tile of grids up to 64 x 64 is in exactly one strip,
the partial-sum kernel's width lookup agrees with the strip, and no strip loads
more tiles per K slab than the tile pairs it replaces."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_strips_cover_the_upper_triangle_once(tmp_path):
    exe = str(tmp_path / "gram_strips_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "times-c_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "gram_strips_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "ALL OK" in r.stdout
