"""The C ABI library on a host without a GPU: it loads, exports every entry point
declared in include/mdz_rheo.h, agrees with the ctypes struct layouts, and fails
with a status (no crash, no CPU fallback) when no device is present."""
import ctypes as C
import os
import re

import pytest

import mdz_rheo as R

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mdz_rheo.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mdz_rheo_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = R.load_library()
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/mdz_rheo.h but not exported"


def test_struct_layouts_match():
    assert R.abi_sizes()[:6] == R.python_struct_sizes()


def test_version_and_status_strings():
    lib = R.load_library()
    assert lib.mdz_rheo_version() == 1
    assert R.status_string(R.MDZ_EVE_ITER) == "Visco-Elastic iterations failed!"
    assert R.status_string(12345) == "unknown status"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU behaviour")
def test_no_device_is_an_error_not_a_fallback():
    with pytest.raises(R.RheoError):
        R.Context(0)
    lib = R.load_library()
    assert lib.mdz_rheo_sweep(None, None, None, None, 0, 0, 0, None) == R.MDZ_EINVAL
