"""Derivation of the float32 polynomial used by ismc_neglog_u32 for
ln(1 + f), f = m - 1, m in [sqrt(1/2), sqrt(2)].

    ln(1 + f) = f - f^2/2 + f^3 * Q(f)

Q is a least-squares fit in high precision at Chebyshev nodes of the interval
(the function (ln(1+f) - f + f^2/2) / f^3 is analytic there), rounded to
float32 and then checked by evaluating the kernel's exact float32 operation
sequence against high-precision logarithms on a dense set of float32 m.

    python ismc_gb300/csrc/fit_log_poly.py      # prints the coefficients
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 50
LO, HI = mp.sqrt(mp.mpf(1) / 2) - 1, mp.sqrt(2) - 1
DEG = 7


def q(f):
    f = mp.mpf(f)
    if abs(f) < mp.mpf("1e-12"):
        return mp.mpf(1) / 3 - f / 4
    return (mp.log1p(f) - f + f * f / 2) / f ** 3


def fit():
    n = 64
    nodes = [(LO + HI) / 2 + (HI - LO) / 2 * mp.cos(mp.pi * (2 * k + 1) / (2 * n)) for k in range(n)]
    A = mp.matrix([[x ** j for j in range(DEG + 1)] for x in nodes])
    b = mp.matrix([q(x) for x in nodes])
    coef = mp.lu_solve(A.T * A, A.T * b)
    return [np.float32(float(c)) for c in coef]


def kernel_ln(m, c):
    """float32 evaluation in the kernel's order (numpy float32 = IEEE single)."""
    f32 = np.float32
    f = (m - f32(1)).astype(np.float32)
    p = np.full_like(f, c[-1])
    for cj in reversed(c[:-1]):
        p = (f32(0) + p * f + cj).astype(np.float32)      # reference only: not fused
    f2 = (f * f).astype(np.float32)
    return (f - f32(0.5) * f2 + f2 * f * p).astype(np.float32)


if __name__ == "__main__":
    c = fit()
    for j, v in enumerate(c):
        print(f"c{j} = {float(v)!r:26} ({np.float32(v).view(np.uint32):#010x})")
    m = np.linspace(float(mp.sqrt(0.5)), float(mp.sqrt(2)), 200001).astype(np.float32)
    got = kernel_ln(m, c).astype(np.float64)
    ref = np.log(m.astype(np.float64))
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    print("max rel err (unfused check):", err.max())
