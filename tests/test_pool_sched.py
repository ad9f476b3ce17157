"""The job pool's admission rule (times-c_gb300/csrc/pool_sched.h) compiled for
the CPU with made-up footprints: a large job at the head of the queue starts
once it has waited past the limit although small jobs keep arriving, and idle
workers hand their workspaces back only when that lets a job start."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pool_head_job_is_not_starved(tmp_path):
    exe = str(tmp_path / "pool_sched_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "times-c_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "pool_sched_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "ALL OK" in r.stdout
