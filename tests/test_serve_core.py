"""CPU checks of the serving policy (queues per database, the continuous-
batching rule, least-recently-used key residency, percentiles) and of the
autotuner's decisions: the C++ headers onionpirv2_gb300/csrc/serve_core.h and
tune_core.h compiled with g++, no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", ["test_serve_core", "test_tune_core"])
def test_host_policy(name):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, name)
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "onionpirv2_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", f"{name}.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
