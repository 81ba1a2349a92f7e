"""The loaded library's kernels were compiled for sm_103a, as the CUDA
runtime reports it for the module it loaded."""
import pytest

from mgmol_gb300 import capi

pytestmark = pytest.mark.gpu


def test_kernels_are_sm103a():
    assert capi.kernel_arch() == 103
