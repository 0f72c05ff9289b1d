"""The reference order's Coulomb forces take the single-precision product
where ChargePotForce (src/model/forcefield.h:87-146) writes
(float)(et2 * (double)d): checked on the host over the whole float range."""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def test_float_products_equal_rounded_double_products(tmp_path):
    exe = tmp_path / "product_rounding_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", str(HERE / "csrc" / "product_rounding_test.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "5000000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
