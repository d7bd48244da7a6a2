"""The restatement of libstdc++'s std::nth_element that selects the reference's
neighbours on tie rows (tapkee_gb300/csrc/nth_select.h), compiled with g++ and
compared on the CPU with std::nth_element itself: identical final arrangements on
tie-heavy, structured and adversarial (heap-select branch) inputs."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "nth_select_check.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


def test_nth_select_equals_libstdcxx():
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "nth_select_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    f"-I{os.path.join(ROOT, 'tapkee_gb300', 'csrc')}", SRC, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"
