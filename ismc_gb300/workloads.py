"""Synthetic workloads of the benchmark set (seeded; no external data).

  bench0_*     one turbid slab between n = 1.5 slides            (1e5 packets)
  bench1_*     three tissue layers between n = 1.52 slides       (1e8 packets)
  lookup_grid  64 x 64 (mu_a, mu_s') single-slab grid with uneven photon budgets
               plus 512 random 1-5 layer stacks                 (one batched launch)
  surrogate_*  uniform samples of (log mu_a, log mu_s', g, d, n)  (training data)
  solve_*      synthetic measurements for the batched inverse solve

Sphere geometry throughout: radius 5.08 cm spheres, sample / entrance ports
of radius 1.27 cm, detector port 0.635 cm, wall reflectance 0.98, both
spheres present (crosstalk on), converted to the reference's port area
fractions by the spherical-cap formula (api.cap_fraction).
"""
import math

import numpy as np

from .api import Layer, Spheres, make_instance

MUA_RANGE = (0.01, 10.0)        # 1/cm
MUSR_RANGE = (1.0, 100.0)       # reduced scattering, 1/cm


def bench_spheres():
    return Spheres.from_radii(5.08, 1.27, 1.27, 0.635, 0.98, R=True, T=True)


def bench0_layers():
    return [Layer.slide(1.5, 0.1), Layer(1.4, 1.0, 100.0, 0.9, 0.1), Layer.slide(1.5, 0.1)]


def bench1_layers():
    return [Layer.slide(1.52, 0.1), Layer(1.37, 0.5, 200.0, 0.8, 0.01),
            Layer(1.40, 2.0, 120.0, 0.9, 0.15), Layer(1.44, 0.2, 50.0, 0.75, 0.3),
            Layer.slide(1.52, 0.1)]


def slab_between_slides(n, mua, mus_reduced, g, d, slide_n=1.5, slide_d=0.1):
    return [Layer.slide(slide_n, slide_d), Layer.from_reduced(n, mua, mus_reduced, g, d),
            Layer.slide(slide_n, slide_d)]


def lookup_grid(seed=2, grid=64, extra=512, budget_range=(1e5, 1e7), scale=1.0):
    """The batched lookup-table generation workload.

    grid x grid single-slab instances: mu_a log-spaced over 0.01-10 1/cm,
    mu_s' log-spaced over 1-100 1/cm, g = 0.9, n = 1.4, d drawn from
    {0.05, 0.1, 0.2} cm, slides n = 1.5 / 0.1 cm, photon budget log-uniform
    over budget_range (times `scale`).  Plus `extra` stacks of 1-5 random
    tissue layers (n in [1.33, 1.5], mu_a and mu_s' log-uniform in the same
    ranges, g = 0.9, d log-uniform over 0.02-0.5 cm) between the same slides.
    Returns (instances, description)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sph = bench_spheres()
    mua = np.geomspace(*MUA_RANGE, grid)
    musr = np.geomspace(*MUSR_RANGE, grid)
    lo, hi = math.log(budget_range[0]), math.log(budget_range[1])
    insts = []
    k = 0
    for i in range(grid):
        for j in range(grid):
            d = float(rng.choice([0.05, 0.1, 0.2]))
            n = max(1, int(round(math.exp(rng.uniform(lo, hi)) * scale)))
            layers = slab_between_slides(1.4, float(mua[i]), float(musr[j]), 0.9, d)
            insts.append(make_instance(layers, sph, n, seed=seed, stream=k, mode="compat"))
            k += 1
    for _ in range(extra):
        nl = int(rng.integers(1, 6))
        layers = [Layer.slide(1.5, 0.1)]
        for _ in range(nl):
            layers.append(Layer.from_reduced(
                float(rng.uniform(1.33, 1.5)),
                float(math.exp(rng.uniform(math.log(MUA_RANGE[0]), math.log(MUA_RANGE[1])))),
                float(math.exp(rng.uniform(math.log(MUSR_RANGE[0]), math.log(MUSR_RANGE[1])))),
                0.9, float(math.exp(rng.uniform(math.log(0.02), math.log(0.5))))))
        layers.append(Layer.slide(1.5, 0.1))
        n = max(1, int(round(math.exp(rng.uniform(lo, hi)) * scale)))
        insts.append(make_instance(layers, sph, n, seed=seed, stream=k, mode="compat"))
        k += 1
    return insts
