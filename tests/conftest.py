import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "svo-tracer_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests through the C ABI")
    # SVO_TEST_WATCHDOG=<seconds>: dump every thread's Python stack periodically
    if os.environ.get("SVO_TEST_WATCHDOG"):
        import faulthandler

        faulthandler.dump_traceback_later(int(os.environ["SVO_TEST_WATCHDOG"]), repeat=True)


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    import build_native
    import build_oracle

    build_native.build()
    build_oracle.build_all()
    yield


@pytest.fixture(scope="session")
def tracer():
    import svo_tracer as st

    tr = st.Tracer(0)
    yield tr
    tr.close()
