import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libug4gb.so")
    config.addinivalue_line("markers", "slow: full-size configurations")


def pytest_sessionfinish(session, exitstatus):
    """UG4GB_GUARD_REPORT (set by tests/test_gpu_guarded.py for its child
    run against the guarded library): write the guard-zone check there"""
    path = os.environ.get("UG4GB_GUARD_REPORT")
    if not path:
        return
    import json
    from ugcore_gb300 import _lib
    n, text = _lib.debug_guard_check()
    with open(path, "w") as fh:
        json.dump({"library": _lib.LIB_PATH, "damaged": n, "report": text, "exitstatus": int(exitstatus)}, fh)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def built_lib():
    from ugcore_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    import ugcore_gb300 as ug
    c = ug.Context(0)
    yield c
    c.close()
