"""The GPU paths against the guarded build of the library.

ugcore's debug builds check every matrix and vector index (UG_ASSERT in
lib_algebra); the device code here is checked instead by a build in which
every device buffer lies between two 4 KB guard zones and starts out as 0xFF
bytes (ugcore_gb300/csrc/guard.cu): a kernel that writes past either end of a
buffer damages a zone, and one that reads memory nobody wrote gets NaN (or -1
as an index), which the parity tests then see.  This test builds that
variant, runs the GPU test files at their small sizes against it in a child
process (UG4GB_LIB_PATH), and requires every test to pass and every zone to
be intact at the end (ug4gb_debug_guard_check, written by tests/conftest.py).
The full-size configurations stay with the normal build.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FILES = ["tests/test_gpu_parity.py", "tests/test_gpu_algebra_ops.py", "tests/test_gpu_conversions.py",
         "tests/test_gpu_fv1_pins.py", "tests/test_gpu_gmg_reinit.py", "tests/test_gpu_io.py",
         "tests/test_gpu_newton.py", "tests/test_gpu_perm.py", "tests/test_gpu_rap.py", "tests/test_gpu_refine.py",
         "tests/test_gpu_sweep_fusion.py", "tests/test_gpu_time_step.py", "tests/test_gpu_unstructured.py",
         "tests/test_gpu_adjoint.py", "tests/test_gpu_coarse_cycle.py", "tests/test_gpu_base_lu.py"]
# full-size cases (193^3 and 129^3 problems) are left to the normal build
SKIP = "not full_size"


def test_gpu_paths_keep_their_buffers(tmp_path):
    from ugcore_gb300 import build
    lib = build.build_guarded(os.path.join(ROOT, "ugcore_gb300", "_build_guarded"))
    report = tmp_path / "guard.json"
    env = dict(os.environ, UG4GB_LIB_PATH=lib, UG4GB_GUARD_REPORT=str(report), PYTHONDONTWRITEBYTECODE="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider", "-k", SKIP] + FILES
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-6000:]
    rep = json.loads(report.read_text())
    assert os.path.samefile(rep["library"], lib)
    assert rep["damaged"] == 0, rep["report"]
    print(out.strip().splitlines()[-1])
