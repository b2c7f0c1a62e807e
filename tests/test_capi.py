"""CPU checks of the C ABI library: it loads, exports every symbol that
include/ismc.h declares, its struct layouts match the ctypes mirror, and it
reports (rather than crashes on) the absence of a GPU."""
import ctypes as C
import os
import re

import pytest

from ismc_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return _abi.declare(C.CDLL(path))


def test_header_and_bindings_agree():
    hdr = open(os.path.join(ROOT, "include", "ismc.h")).read()
    declared = set(re.findall(r"^\s*(?:int|size_t)\s+(ismc_\w+)\s*\(", hdr, re.M))
    assert declared == set(_abi.EXPORTS), declared ^ set(_abi.EXPORTS)


def test_exports_and_layout(lib):
    for name in _abi.EXPORTS:
        assert hasattr(lib, name), name
    for k, cls in _abi.SIZEOF_INDEX.items():
        assert lib.ismc_sizeof(k) == C.sizeof(cls)
    assert lib.ismc_version() == _abi.ABI_VERSION


def test_errors_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.ismc_init(0, C.byref(h))
    assert rc == _abi.ERR_NO_DEVICE
    buf = C.create_string_buffer(256)
    assert lib.ismc_last_error(None, buf, 256) == 0
    assert b"no CUDA device" in buf.value
    assert lib.ismc_init(0, None) == _abi.ERR_INVALID_ARG
    assert lib.ismc_run(None, None, None, 0, 0, 0, None) == _abi.ERR_INVALID_ARG
    assert lib.ismc_run_batch(None, None, 0, None, None) == _abi.ERR_INVALID_ARG
