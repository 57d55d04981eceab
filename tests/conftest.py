import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
REF_MODULES = ["DD", "DDrppi", "DDsmu", "wp", "xi", "DDtheta"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


def ref_lib_path(name):
    return os.path.join(REF_DIR, "libcf_ref_%s.so" % name)


def have_reference():
    return all(os.path.exists(ref_lib_path(m)) for m in REF_MODULES)


@pytest.fixture(scope="session")
def reflibs():
    """ctypes handles of the reference's own pair counters compiled into oracle/_ref."""
    if not have_reference():
        pytest.skip("reference libraries not built in oracle/_ref")
    from corrfunc_gb300 import _capi as C
    return {m: C.bind(ref_lib_path(m)) for m in REF_MODULES}


# reference modules that include GSL headers, compiled against the test-only stand-in
REF_GSL_MODULES = ["DDrppi_mocks", "DDsmu_mocks", "vpf", "vpf_mocks"]


@pytest.fixture(scope="session")
def reflibs_gsl():
    """ctypes handles of the reference's survey counters and counts-in-spheres modules (oracle/_ref,
    built against the GSL stand-in in oracle/gsl_shim)."""
    if not all(os.path.exists(ref_lib_path(m)) for m in REF_GSL_MODULES):
        pytest.skip("reference survey / vpf libraries not built in oracle/_ref")
    from corrfunc_gb300 import _capi as C
    return {m: C.bind(ref_lib_path(m)) for m in REF_GSL_MODULES}


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
