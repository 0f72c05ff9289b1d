"""The reference-side binding (host/reference/GB300EnergyService6D.h) compiles
inside the reference tree against its own Service / EnergyService / Server
headers, in the reference's language level (C++11) and CUDA configuration.
Runs where the reference sources are present; skipped elsewhere."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _ref_src():
    import sys
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle
    r = pyoracle.ref_root()
    return None if r is None else r / "src"


REF = _ref_src()

SNIPPET = r'''
#include "GB300EnergyService6D.h"
#include "Server.h"
template class as::Server<as::Types_6D<float>>;
void use(std::shared_ptr<as::DataManager> dm) {
	auto s = std::make_shared<as::GB300EnergyService6D>(dm);
	as::Server<as::Types_6D<float>> srv(s);
	srv.createWorkers(2);
}
'''


@pytest.mark.skipif(REF is None, reason="reference sources not present on this host")
def test_binding_compiles_against_reference(tmp_path):
    src = tmp_path / "bind.cpp"
    src.write_text(SNIPPET)
    inc = []
    for d in sorted(p for p in REF.rglob("*") if p.is_dir() and len(p.relative_to(REF).parts) <= 2):
        inc += ["-I", str(d)]
    cmd = ["g++", "-std=c++11", "-DCUDA", "-fsyntax-only", "-I", str(REF), *inc,
           "-I", str(ROOT / "gpuattract_2.0_gb300" / "host" / "reference"), "-I", str(ROOT / "include"),
           "-I", "/usr/local/cuda/include", str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
