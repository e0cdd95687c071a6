"""The C++ drop-in (include/onionpir_server.hpp) runs the reference's
test_pir loop (src/tests.cpp:40-153) end to end through the C ABI."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_pir_server_round_trip(oracle_lib, gpu_lib):
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_pir_server")
    gpu_dir = os.path.join(ROOT, "onionpirv2_gb300", "_build")
    orc_dir = os.path.join(ROOT, "oracle", "_build")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "cpp", "test_pir_server.cpp"),
           "-o", exe, f"-L{gpu_dir}", "-lopir_gb300", f"-L{orc_dir}", "-lopir_oracle",
           f"-Wl,-rpath,{gpu_dir}", f"-Wl,-rpath,{orc_dir}"]
    # the libraries are built as lib*.so in their _build folders
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Success rate: 13/13, bit-identical: 13/13" in r.stdout
    assert "batch == single: 13/13, served == single: 13/13" in r.stdout
