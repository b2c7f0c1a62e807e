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


def test_header_constants_match_bindings():
    hdr = open(os.path.join(ROOT, "include", "ismc.h")).read()

    def define(name):
        m = re.search(r"^#define\s+" + name + r"\s+(\S+)", hdr, re.M)
        assert m, name
        return int(m.group(1).rstrip("uUlL").strip("()"), 0)
    assert define("ISMC_NOALLOC_MAX_INST") == _abi.NOALLOC_MAX_INST
    assert define("ISMC_MAX_PACKETS") == _abi.MAX_PACKETS
    assert define("ISMC_MAXL") == _abi.MAXL
    assert define("ISMC_ABI_VERSION") == _abi.ABI_VERSION
    for code, name in _abi.ERR_NAMES.items():
        if code:
            assert define("ISMC_ERR_" + name) == code, name


def test_validate_refuses_without_a_launch(lib):
    """Host-side checks need no GPU: an instance claiming more packets than
    64-bit tallies can hold (5e9 > 2^31) is refused with ISMC_ERR_CAPACITY,
    the limit itself is accepted, and a bad roulette is an invalid argument."""
    from ismc_gb300 import Layer, Spheres, make_instance
    good = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], Spheres(), _abi.MAX_PACKETS, seed=1)
    big = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], Spheres(), 5_000_000_000, seed=1)
    roul = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], Spheres(), 10, seed=1,
                         roulette_threshold=0.5, roulette_m=10.0)
    arr = (_abi.Instance * 3)(good, big, roul)
    st = (C.c_int32 * 3)()
    rc = lib.ismc_validate(arr, 3, st)
    assert rc == _abi.ERR_CAPACITY
    assert list(st) == [_abi.OK, _abi.ERR_CAPACITY, _abi.ERR_INVALID_ARG]
    buf = C.create_string_buffer(512)
    lib.ismc_last_error(None, buf, 512)
    assert b"5000000000 packets exceed" in buf.value
    assert lib.ismc_validate(arr, 1, None) == _abi.OK


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


def test_integration_cpp_shim_compiles(tmp_path):
    """The C++ shim INTEGRATION.md gives the reference's CUDA callers (the
    ISMLMC() signature of CUDA/CUDAISMLMC.h:656 over ismc_run) compiles
    against include/ismc.h."""
    import shutil
    import subprocess
    with open(os.path.join(ROOT, "INTEGRATION.md")) as fh:
        blocks = re.findall(r"```cpp\n(.*?)```", fh.read(), re.S)
    assert blocks
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if shutil.which("g++") is None or not os.path.isdir(os.path.join(cuda_inc, "cccl")):
        pytest.skip("g++ or the CUDA toolkit's thrust headers are absent")
    src = tmp_path / "shim.cpp"
    src.write_text(blocks[0])
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"),
                        "-I" + cuda_inc, "-I" + os.path.join(cuda_inc, "cccl"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
