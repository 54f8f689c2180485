import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def golden_files():
    with open(os.path.join(GOLDEN, "golden_factor_files.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build

    build.build_oracle()
    import oracle

    return oracle


@pytest.fixture(scope="session")
def eng():
    """The GPU engine (GPU tests only)."""
    import cutrialdive_gb300 as ctd

    return ctd.engine(0)
