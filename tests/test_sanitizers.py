"""The host code under AddressSanitizer and UndefinedBehaviorSanitizer.

ugcore's own test strategy runs its unit tests under valgrind and the
compilers' sanitizers; the counterpart here is a build of the same sources
with -fsanitize=address,undefined in the host code:

  - the oracle (oracle/liboracle_asan.so, `make -C oracle liboracle_asan.so`)
    running its golden-vector tests and the FV1 geometry pins;
  - the library (ugcore_gb300/_build_asan/libug4gb_asan.so,
    ugcore_gb300.build.build_sanitized) running the host-only tests: the
    MatrixMarket / ConnectionViewer / UGX readers and writers on the golden
    files and on malformed inputs, the C-ABI argument checks, the hierarchy
    set-up.

Each runs in a child pytest with the sanitizer runtimes preloaded (python
itself is not instrumented); any report fails the test.  No GPU is used:
device code is compiled as usual but not run.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _runtime(name):
    try:
        p = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    except OSError:
        return None
    return p if os.path.isabs(p) and os.path.exists(p) else None


def _child(tests, env_extra, timeout):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("gcc's sanitizer runtimes are not installed")
    env = dict(os.environ)
    env.update(env_extra)
    env["LD_PRELOAD"] = asan + ":" + ubsan
    # leaks: python and the CUDA runtime keep allocations to the end;
    # the CUDA runtime maps the address range ASan keeps as a shadow gap
    env["ASAN_OPTIONS"] = "detect_leaks=0:protect_shadow_gap=0:abort_on_error=0:halt_on_error=1"
    env["UBSAN_OPTIONS"] = "print_stacktrace=1:halt_on_error=1"
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "not gpu", "-p", "no:cacheprovider"] + tests
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-4000:]
    for word in ("AddressSanitizer", "runtime error:", "LeakSanitizer"):
        assert word not in out, out[-4000:]
    return out


def test_oracle_under_sanitizers():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle_asan.so"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = os.path.join(ROOT, "oracle", "liboracle_asan.so")
    out = _child(["tests/test_oracle.py", "tests/test_fv1_pins.py"], {"UG4GB_ORACLE_LIB": lib}, 900)
    assert " passed" in out


def test_library_host_code_under_sanitizers():
    from ugcore_gb300 import build
    lib = build.build_sanitized(os.path.join(ROOT, "ugcore_gb300", "_build_asan"))
    tests = ["tests/test_io.py", "tests/test_grids.py", "tests/test_abi.py::test_calls_without_device_return_status"]
    out = _child(tests,
                 {"UG4GB_LIB_PATH": lib}, 900)
    assert " passed" in out
