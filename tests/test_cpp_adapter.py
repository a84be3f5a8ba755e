"""The header-only C++ adapter (include/lustrine_gb300_sim.hpp) compiles and
links against liblustrine_gb300.so with the reference's Simulation fields,
and its function has the reference's step-hook signature.  Compile-time
only: no GPU call."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = "/root/reference"


def _compile(tmp_path, extra):
    from lustrine_gb300 import _lib
    lib = _lib.load()  # builds the library if needed
    out = tmp_path / "adapter_check"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), *extra,
           os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"), "-o", str(out),
           _lib.library_path(), "-Wl,-rpath," + os.path.dirname(_lib.library_path())]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert lib is not None
    return out


def test_adapter_compiles_with_simulation_fields(tmp_path):
    _compile(tmp_path, [])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference tree not mounted")
def test_adapter_compiles_against_reference_simulation(tmp_path):
    shim = os.path.join(ROOT, "oracle", "ref_shim")
    _compile(tmp_path, ["-DWITH_REFERENCE", "-DPLATFORM_UNIX", "-w", "-I", shim, "-I", f"{REF}/src",
                        "-I", f"{REF}/thirdparty/glm-0.9.9.8", "-I", f"{REF}/thirdparty/Bullet3/bullet3/src",
                        "-c"])
