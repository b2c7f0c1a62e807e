"""ORACLE -- test infrastructure only.

Nothing in the product imports this package.  Only tests/, the smoke check of
__graft_entry__.py and bench.py's CPU-baseline / reference arm use it, and only
as the checker or as the timed CPU baseline, never as the measured GPU path.

Contents
  twin_run      FP32 C restatement of the GPU event algorithm, same Philox
                streams: must equal the GPU's integer tallies bit for bit.
  ref64_run     FP64 C restatement of the reference's ISMC.py / ISMLMC.py
                structure (statistical oracle and CPU baseline), with an FP64
                walk of the kernel's physical mode for instances in that mode.
  build_ref / refpython  the reference's own sources staged into oracle/_ref/
                (PRAXIS, the CUDA model, the drivers, the Python model) and a
                process pool that runs the staged ISMLMC.py.
  analytic64    FP64 specular / ballistic values of a stack (oracle/analytic64.py).
  golden_cases  statistical fixtures produced by the reference's own Python
                (tests/golden/reference_cases.json, made by tests/golden/make_golden.py).
"""
import ctypes as C
import json
import math
import os

from ismc_gb300 import _abi
from . import build as _build
from .analytic64 import analytic64  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden", "reference_cases.json")
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(_build.build())
        P = C.POINTER
        L.twin_run.restype = C.c_int
        L.twin_run.argtypes = [P(_abi.Instance), C.c_uint32, C.c_int, P(_abi.Tally)]
        L.twin_packet.restype = C.c_int
        L.twin_packet.argtypes = [P(_abi.Instance), C.c_uint64, C.c_uint32, P(C.c_float),
                                  P(C.c_float), P(C.c_int), P(C.c_uint32)]
        L.twin_philox.restype = None
        L.twin_philox.argtypes = [P(C.c_uint32), C.c_uint32, C.c_uint32, P(C.c_uint32)]
        L.twin_u01.restype = C.c_float
        L.twin_u01.argtypes = [C.c_uint32]
        L.twin_neglog_u32.restype = C.c_float
        L.twin_neglog_u32.argtypes = [C.c_uint32]
        L.twin_sincos_2pi.restype = None
        L.twin_sincos_2pi.argtypes = [C.c_float, P(C.c_float), P(C.c_float)]
        L.twin_expneg.restype = C.c_float
        L.twin_expneg.argtypes = [C.c_float]
        L.twin_fresnel.restype = C.c_float
        L.twin_fresnel.argtypes = [C.c_float, C.c_float, P(C.c_float)]
        L.twin_fresnel_reflects.restype = C.c_int
        L.twin_fresnel_reflects.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        L.ref64_run.restype = C.c_int
        L.ref64_run.argtypes = [C.c_int, P(_abi.Instance), C.c_int, P(C.c_double),
                                P(C.c_double), P(C.c_uint64)]
        _LIB = L
    return _LIB


def twin_run(inst, threads=None, max_events=0):
    """Integer tallies of the FP32 twin for one ABI instance (threads never
    change the result)."""
    out = _abi.Tally()
    rc = lib().twin_run(C.byref(inst), max_events, threads or os.cpu_count(), C.byref(out))
    if rc:
        raise ValueError("twin_run rejected the instance")
    return out


def ref64_run(inst, single=False, threads=None):
    """FP64 restatement of the reference; returns (mean[5], se[5], steps)."""
    s = (C.c_double * 5)()
    q = (C.c_double * 5)()
    steps = C.c_uint64()
    rc = lib().ref64_run(1 if single else 0, C.byref(inst), threads or os.cpu_count(), s, q,
                         C.byref(steps))
    if rc:
        raise ValueError("ref64_run rejected the instance")
    n = inst.n_packets
    mean = [s[k] / n for k in range(5)]
    se = [math.sqrt(max(q[k] / n - mean[k] ** 2, 0.0) / (n - 1)) if n > 1 else 0.0
          for k in range(5)]
    return mean, se, int(steps.value)


def golden_cases():
    with open(GOLDEN) as fh:
        return json.load(fh)["cases"]
