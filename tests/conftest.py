import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built extension")


@pytest.fixture(scope="session")
def test_cosmology():
    """The cosmology of the reference's own tests (tests/test_perturbations.py:11-57)."""
    import discoeb_gb300.background as bg
    from discoeb_gb300.workloads import reference_test_param

    return bg.evolve_background(param=reference_test_param())
