import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built library")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref_lib():
    import oracle

    if oracle.ref_dir() is None and not oracle.ref_available():
        pytest.skip("DEMON_REF_DIR not set and no compiled reference in oracle/_ref")
    if oracle.ref_dir() is not None:
        try:
            oracle.build(ref=True)
        except Exception as e:  # not x86-64
            pytest.skip(f"reference not buildable here: {e}")
    if not oracle.ref_available():
        pytest.skip("reference library not built")
    return oracle.Reference()


@pytest.fixture(scope="session")
def gpu_ctx():
    from demon_simulation_code_gb300 import Context, load

    load()
    return Context(0)
