import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "webgraph-algo-rs_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")
# cnr-2000 BVGraph copies made by tests/golden/make_fixtures.py (git-ignored,
# shipped with the working tree); a reference checkout named by the
# HB_REFERENCE environment variable is searched after them.
_REF = os.environ.get("HB_REFERENCE")
CNR_DIRS = [os.path.join(GOLDEN, "_data")] + (
    [os.path.join(_REF, "tests", "graphs")] if _REF else [])
CNR_RESULTS_DIRS = [os.path.join(GOLDEN, "_data")] + (
    [os.path.join(_REF, "tests", "hyperball_results")] if _REF else [])


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def _find(dirs, name):
    for d in dirs:
        p = os.path.join(d, name)
        if os.path.exists(p):
            return p
    return None


def cnr_basename(transpose=False):
    name = "cnr-2000-t" if transpose else "cnr-2000"
    p = _find(CNR_DIRS, name + ".graph")
    return p[: -len(".graph")] if p else None


def cnr_result(name):
    return _find(CNR_RESULTS_DIRS, "cnr-2000_" + name)


@pytest.fixture(scope="session")
def product_lib():
    import build_lib

    build_lib.build()
    import hyperball_gb300 as hb

    return hb.load_library()


@pytest.fixture(scope="session")
def hb(product_lib):
    import hyperball_gb300

    return hyperball_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import hbo

    hbo.lib()
    return hbo
