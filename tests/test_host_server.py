"""The C++ request interface (gpuattract_2.0_gb300/host/gba_server.h) against
the reference's own server test cases, with mock services (no GPU)."""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def test_server_interface_and_sweep(tmp_path):
    exe = tmp_path / "server_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", str(HERE / "csrc" / "server_test.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "OK"
