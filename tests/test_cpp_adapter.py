"""The header-only C++ adapter (include/lustrine_gb300_sim.hpp) compiles and
links against liblustrine_gb300.so with the reference's Simulation fields,
and its function has the reference's step-hook signature (compile-time, no
GPU call); on the GPU, it steps a Simulation-shaped struct exactly as the
context API does while the sand count changes between steps."""
import os
import subprocess

import pytest

from conftest import HAVE_REF, REF, ROOT


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


@pytest.mark.skipif(not HAVE_REF, reason="LUSTRINE_REFERENCE_DIR not set")
def test_adapter_compiles_against_reference_simulation(tmp_path):
    shim = os.path.join(ROOT, "oracle", "ref_shim")
    _compile(tmp_path, ["-DWITH_REFERENCE", "-DPLATFORM_UNIX", "-w", "-I", shim, "-I", f"{REF}/src",
                        "-I", f"{REF}/thirdparty/glm-0.9.9.8", "-I", f"{REF}/thirdparty/Bullet3/bullet3/src",
                        "-c"])


@pytest.mark.gpu
def test_adapter_steps_match_context_api_while_sand_count_changes(tmp_path):
    import numpy as np
    from lustrine_gb300 import PbfSim, _lib, reference_params
    lib = _lib.load()
    exe = tmp_path / "adapter_run"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_run.cpp"), "-o", str(exe),
           _lib.library_path(), "-Wl,-rpath," + os.path.dirname(_lib.library_path())]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = tmp_path / "states.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    raw = np.fromfile(out, dtype=np.uint8)
    off, counts = 0, []

    def take(k, dtype):
        nonlocal off
        a = np.frombuffer(raw[off:off + 4 * k].tobytes(), dtype=dtype)
        off += 4 * k
        return a

    while off < len(raw):
        n, ns = (int(a) for a in take(2, np.int32))
        x_in, v_in = take(3 * n, np.float32).reshape(n, 3), take(3 * n, np.float32).reshape(n, 3)
        solid = take(3 * ns, np.float32).reshape(ns, 3)
        x_out, v_out = take(3 * n, np.float32).reshape(n, 3), take(3 * n, np.float32).reshape(n, 3)
        sim = PbfSim(reference_params(24, 24, 24, 0.5, 2.0), n, ns)
        sim.upload(x_in, v_in, solid)
        sim.step(1 / 60)
        x, v, _, _ = sim.download()
        sim.close()
        np.testing.assert_array_equal(x, x_out)
        np.testing.assert_array_equal(v, v_out)
        counts.append(n)
    assert counts == [512, 512, 522, 492, 1092]
    assert lib is not None


@pytest.mark.gpu
def test_sand_adapter_steps_match_oracle_while_sand_count_changes(tmp_path, orc):
    """simulate_sand<Simulation> on a Simulation-shaped struct (attract in
    steps 1-2, blow in step 3, the sand count changing between steps): every
    step equals the oracle's restatement of the reference's sand step, flags
    included."""
    import numpy as np
    from lustrine_gb300 import _lib
    lib = _lib.load()
    exe = tmp_path / "adapter_run"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_run.cpp"), "-o", str(exe),
           _lib.library_path(), "-Wl,-rpath," + os.path.dirname(_lib.library_path())]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = tmp_path / "states.bin"
    r = subprocess.run([str(exe), str(out), "sand"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    raw = np.fromfile(out, dtype=np.uint8)
    off, counts = 0, []

    def take(k, dtype):
        nonlocal off
        a = np.frombuffer(raw[off:off + 4 * k].tobytes(), dtype=dtype)
        off += 4 * k
        return a

    p = orc.reference_params(24, 24, 24, 0.5, 2.0)  # rest density 24, mass 5, gravity -10
    prev, k, seen = False, 0, 0
    while off < len(raw):
        n, ns = (int(a) for a in take(2, np.int32))
        x_in, v_in = take(3 * n, np.float32).reshape(n, 3), take(3 * n, np.float32).reshape(n, 3)
        solid = take(3 * ns, np.float32).reshape(ns, 3)
        att_in = take(n, np.int32)
        x_out, v_out = take(3 * n, np.float32).reshape(n, 3), take(3 * n, np.float32).reshape(n, 3)
        att_out = take(n, np.int32)
        attract, blow = k in (1, 2), k == 3
        ctl = orc.sand_controls(player=(10.0, 8.0, 10.0), attract=attract, blow=blow, prev_attract=prev,
                                diameter=1.0)
        o = orc.sand_step(p, ctl, np.float32(1 / 60), x_in, v_in, att_in, solid=solid, cap=96)
        np.testing.assert_array_equal(o["x"], x_out)
        np.testing.assert_array_equal(o["v"], v_out)
        np.testing.assert_array_equal(o["attracted"], att_out)
        seen = max(seen, int(att_out.sum()))
        prev = attract
        counts.append(n)
        k += 1
    assert counts == [512, 512, 522, 492, 1092]
    assert seen > 0
    assert lib is not None
