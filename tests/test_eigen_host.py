"""The eigensolver's host linear algebra (tapkee_gb300/csrc/eigen_host.h: Cholesky,
triangular inverse, cyclic Jacobi), compiled with g++ and run on the CPU."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "eigen_host_check.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


def test_eigen_host_linear_algebra():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "eigen_host_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    f"-I{os.path.join(ROOT, 'tapkee_gb300', 'csrc')}", SRC, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"
