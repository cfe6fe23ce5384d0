import pathlib
import sys

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "tests"))
sys.path.insert(0, str(REPO / "thesis-emx-bach_gb300"))


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300, sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    import build_native
    build_native.build_oracle()
    from xbach_testlib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def test01():
    from xbach_testlib import GOLDEN, read_fits
    return {
        "S": read_fits(GOLDEN / "test0.fits"),   # science (-s test0)
        "T": read_fits(GOLDEN / "test1.fits"),   # template (-t test1)
        "conv": read_fits(GOLDEN / "test01_conv.fits"),
        "sub": read_fits(GOLDEN / "test01_sub.fits"),
    }


@pytest.fixture(scope="session")
def test01_oracle(oracle, test01):
    return oracle.run(oracle.default_params(), test01["T"], test01["S"])
