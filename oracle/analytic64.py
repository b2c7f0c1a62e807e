"""ORACLE: FP64 deterministic quantities of a layer stack (test infrastructure).

Inputs are the stack's FP32 values (promoted exactly to FP64), so the only
difference from the GPU's values is the GPU's arithmetic.

specular (normal incidence)
  compatible mode: the incidence series of ISMLMC.py:79-93,
      R = r1 + (1 - r1)^2 r2 / (1 - r1 r2)   when the top layer is a slide
                                              (mu_s == 0, ISMLMC.py:81),
      R = r1                                  otherwise,
    with r1 = Fresnel(ambient -> n0), r2 = Fresnel(n0 -> n1) at normal incidence,
    i.e. ((a - b)/(a + b))^2 (the |mu_z| > 0.99999 branch of MLMC.py:46).
  physical mode: reflectance, seen from the ambient, of the incoherent stack of
    every interface and slide above the first scattering layer.
ballistic: transmittance of the incoherent stack of every interface and layer,
  each layer attenuating unscattered light by exp(-mu_t d).

Incoherent stacking of a symmetric element (r, t) below a composite with
front/back reflectance Rf/Rb and transmittance Tf/Tb:
  D = 1 - Rb r;  Rf += Tf Tb r / D;  Tf *= t / D;  Rb = r + t^2 Rb / D;  Tb *= t / D.
"""
import math

import numpy as np


def _f64(x):
    return float(np.float32(x))


def _r0(a, b):
    return ((a - b) / (a + b)) ** 2


def _add(S, r, t):
    Rf, Tf, Rb, Tb = S
    D = 1.0 - Rb * r
    return (Rf + Tf * Tb * r / D, Tf * t / D, r + t * t * Rb / D, Tb * t / D)


def analytic64(n, mus, mut, d, mode="compat"):
    """(specular, ballistic) of a stack given per-layer n, mu_s, mu_t, d."""
    n = [_f64(x) for x in n]
    mus = [_f64(x) for x in mus]
    mut = [_f64(x) for x in mut]
    d = [_f64(x) for x in d]
    L = len(n)
    spec = None
    if mode == "compat":
        r1 = _r0(1.0, n[0])
        spec = r1
        if mus[0] == 0.0:
            r2 = _r0(n[0], n[1] if L > 1 else 1.0)
            spec = r1 + (1 - r1) ** 2 * r2 / (1 - r1 * r2)
    S = (0.0, 1.0, 0.0, 1.0)
    n_prev = 1.0
    for l in range(L):
        r = _r0(n_prev, n[l])
        S = _add(S, r, 1.0 - r)
        if mus[l] != 0.0 and spec is None:
            spec = S[0]
        S = _add(S, 0.0, math.exp(-mut[l] * d[l]))
        n_prev = n[l]
    r = _r0(n_prev, 1.0)
    S = _add(S, r, 1.0 - r)
    if spec is None:
        spec = S[0]
    return spec, S[1]
