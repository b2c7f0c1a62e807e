"""The allocation-free batch entry point, ismc_run_batch_noalloc.

It serves callers that may not allocate GPU memory themselves or through a
library: a plugin inside an application that owns all device memory, a hard
memory budget, or a latency-critical loop. They pass device-resident
instances and a device-resident tally array; the library works only in its
fixed __device__ array.

The test calls it twice in a row through the C ABI, on the same inputs the
existing device-pointer entry point (ismc_run_batch_device) gets, and requires
the same tallies. Tallies are integer sums, so the parity tests' tolerance
for them is exact equality. The second call shows that state left in the
shared array by the first call does not leak into the next result. This file
sorts last so that a run stopping at the first failure has run everything
else; it also passes on its own in a fresh process.
"""
import ctypes as C

import pytest

import cases
from ismc_gb300 import _abi, build, load_library, make_tune

pytestmark = pytest.mark.gpu


def _tallies(buf, n):
    return (_abi.Tally * n).from_buffer_copy(buf.cpu().numpy().tobytes())


def _key(t):
    return (list(t.sum), list(t.sumsq), t.steps, t.events, t.reincidences, t.capped, t.trapped,
            t.n, t.status, t.analytic_specular, t.analytic_ballistic)


def test_noalloc_matches_device_entry_twice():
    import torch
    from ismc_gb300 import Engine
    build.build()
    lib = load_library()
    G = cases.golden()
    insts = [cases.case_instance(G[name], n, seed=900 + k, stream=k)
             for k, (name, n) in enumerate([("bench0_slides", 40_000), ("bench1_multilayer", 7_000),
                                            ("slab_both", 0), ("five_layer_mixed", 12_345),
                                            ("grid_low_albedo_thin", 25_000)])]
    n = len(insts)
    raw = bytes((_abi.Instance * n)(*insts))
    d_in = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    size = n * C.sizeof(_abi.Tally)
    ref = torch.zeros(size, dtype=torch.uint8, device="cuda")
    out1 = torch.full((size,), 0xAB, dtype=torch.uint8, device="cuda")
    out2 = torch.full((size,), 0xCD, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    with Engine(0) as eng:
        eng.run_batch_device(d_in.data_ptr(), n, ref.data_ptr(), stream.cuda_stream)
    for out in (out1, out2):
        rc = lib.ismc_run_batch_noalloc(C.c_void_p(d_in.data_ptr()), n, None,
                                        C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0
    stream.synchronize()
    want = [_key(t) for t in _tallies(ref, n)]
    assert [_key(t) for t in _tallies(out1, n)] == want
    assert [_key(t) for t in _tallies(out2, n)] == want
    assert all(t[8] == 0 for t in want)

    # a launch shape of the caller's choosing gives the same integer tallies
    rc = lib.ismc_run_batch_noalloc(C.c_void_p(d_in.data_ptr()), n, C.byref(make_tune(128, 0, 96, 0)),
                                    C.c_void_p(out1.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    assert [_key(t) for t in _tallies(out1, n)] == want


def test_noalloc_full_capacity_batch():
    """Exactly ISMC_NOALLOC_MAX_INST instances: every slot of the fixed array
    (and the last prefix word) is used, and the prefix scan gives each of its
    threads one instance.  Small uneven instances tile the golden cases."""
    import numpy as np
    import torch
    from ismc_gb300 import Engine
    lib = load_library()
    G = cases.golden()
    names = sorted(G)
    rng = np.random.default_rng(11)
    n = _abi.NOALLOC_MAX_INST
    insts = [cases.case_instance(G[names[k % len(names)]], int(rng.integers(0, 400)), seed=31,
                                 stream=k, mode="physical" if k % 5 == 0 else "compat")
             for k in range(n)]
    raw = bytes((_abi.Instance * n)(*insts))
    d_in = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    size = n * C.sizeof(_abi.Tally)
    ref = torch.zeros(size, dtype=torch.uint8, device="cuda")
    out = torch.full((size,), 0x5A, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    with Engine(0) as eng:
        eng.run_batch_device(d_in.data_ptr(), n, ref.data_ptr(), stream.cuda_stream)
    rc = lib.ismc_run_batch_noalloc(C.c_void_p(d_in.data_ptr()), n, None,
                                    C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    want = [_key(t) for t in _tallies(ref, n)]
    assert [_key(t) for t in _tallies(out, n)] == want
    assert sum(t[7] for t in want) == sum(int(x.n_packets) for x in insts)


def test_noalloc_rejects_batches_beyond_capacity():
    lib = load_library()
    rc = lib.ismc_run_batch_noalloc(C.c_void_p(16), _abi.NOALLOC_MAX_INST + 1, None, C.c_void_p(16),
                                    None)
    assert rc == _abi.ERR_CAPACITY
    buf = C.create_string_buffer(512)
    lib.ismc_last_error(None, buf, 512)
    assert b"capacity" in buf.value
