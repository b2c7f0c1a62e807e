"""PRAXIS (Brent's principal-axis method) of the library, on the host, against
known minima and against the reference's own praxis.cpp (built from the
reference checkout into oracle/_ref/ when it is available)."""
import ctypes as C
import math
import os

import pytest

from ismc_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    return _abi.declare(C.CDLL(build.build()))


def ref_lib():
    from oracle import build_ref
    path = build_ref.build()
    if not path:
        return None
    L = C.CDLL(path)
    L.ref_praxis.restype = C.c_double
    L.ref_praxis.argtypes = [_abi.OBJECTIVE, C.c_void_p, C.c_int, C.POINTER(C.c_double),
                             C.c_double, C.c_double, C.POINTER(C.c_int)]
    return L


def rosenbrock(x):
    return 100 * (x[1] - x[0] ** 2) ** 2 + (1 - x[0]) ** 2


def ill_quadratic(x):      # condition number 1e6, rotated axes
    u, v = (x[0] + x[1]) / math.sqrt(2), (x[0] - x[1]) / math.sqrt(2)
    return 1e3 * (u - 1) ** 2 + 1e-3 * (v + 2) ** 2


def powell_singular(x):
    return ((x[0] + 10 * x[1]) ** 2 + 5 * (x[2] - x[3]) ** 2 + (x[1] - 2 * x[2]) ** 4 +
            10 * (x[0] - x[3]) ** 4)


def helix(x):
    th = math.atan2(x[1], x[0]) / (2 * math.pi)
    return 100 * ((x[2] - 10 * th) ** 2 + (math.hypot(x[0], x[1]) - 1) ** 2) + x[2] ** 2


PROBLEMS = [
    ("rosenbrock", rosenbrock, [-1.2, 1.0], [1.0, 1.0]),
    ("ill_quadratic", ill_quadratic, [0.0, 0.0], [1 / math.sqrt(2) * (1 - 2) + 0.0, None]),
    ("powell_singular", powell_singular, [3.0, -1.0, 0.0, 1.0], [0.0, 0.0, 0.0, 0.0]),
    ("helix", helix, [-1.0, 0.0, 0.0], [1.0, 0.0, 0.0]),
]


def _run(fn, f, x0, t0=1e-7, h0=1.0):
    cb = _abi.OBJECTIVE(lambda p, n, u: f([p[i] for i in range(n)]))
    x = (C.c_double * len(x0))(*x0)
    return fn(cb, x, t0, h0), list(x)


@pytest.mark.parametrize("name,f,x0,_", PROBLEMS)
def test_praxis_reaches_known_minimum(lib, name, f, x0, _):
    fmin = C.c_double()
    nf = C.c_int()

    def call(cb, x, t0, h0):
        assert lib.ismc_praxis(cb, None, len(x0), x, t0, h0, 20000, C.byref(fmin), C.byref(nf)) == 0
        return fmin.value
    v, x = _run(call, f, x0)
    assert v < 1e-8, (name, v, x, nf.value)
    assert nf.value < 5000


@pytest.mark.parametrize("name,f,x0,_", PROBLEMS)
def test_praxis_vs_reference_praxis(lib, name, f, x0, _):
    R = ref_lib()
    if R is None:
        pytest.skip("reference checkout not available")
    nf_ref = C.c_int()
    v_ref, x_ref = _run(lambda cb, x, t0, h0: R.ref_praxis(cb, None, len(x0), x, t0, h0,
                                                          C.byref(nf_ref)), f, x0)
    fmin, nf = C.c_double(), C.c_int()
    v, x = _run(lambda cb, xx, t0, h0: (lib.ismc_praxis(cb, None, len(x0), xx, t0, h0, 20000,
                                                        C.byref(fmin), C.byref(nf)),
                                        fmin.value)[1], f, x0)
    # both find the minimum; ours needs no more than twice the evaluations
    assert v_ref < 1e-8 and v < 1e-8, (v_ref, v)
    assert nf.value <= 2 * nf_ref.value + 50, (nf.value, nf_ref.value)
