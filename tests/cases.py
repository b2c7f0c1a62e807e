"""Shared workload definitions for the tests (CPU and GPU).

Golden cases come from tests/golden/reference_cases.json, produced by the
reference's own Python (tests/golden/make_golden.py).  A case's driver decides
the roulette threshold: ISMC.py's single-slab walk uses 1e-3 (ISMC.py:136),
ISMLMC.py's multilayer walk 1e-4 (MLMC.py:86).
"""
import json
import math
import os

from ismc_gb300 import Layer, Spheres, make_instance

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_cases.json")


def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)["cases"]


def case_layers(case):
    return [Layer(L["n"], L["mua"], L["mus"], L["g"], L["d"]) for L in case["layers"]]


def case_spheres(case):
    s = dict(case["spheres"])
    return Spheres(**s)


def case_instance(case, n_packets, seed, mode="compat", stream=0, packet_offset=0):
    thr = 1e-3 if case["driver"] == "ISMC" else 1e-4
    return make_instance(case_layers(case), case_spheres(case), n_packets, seed=seed,
                         stream=stream, mode=mode, roulette_threshold=thr, roulette_m=10.0,
                         packet_offset=packet_offset)


def zscores(mean_a, se_a, mean_b, se_b):
    out = []
    for a, sa, b, sb in zip(mean_a, se_a, mean_b, se_b):
        s = math.sqrt(sa * sa + sb * sb)
        out.append(0.0 if s == 0 and a == b else (a - b) / s if s > 0 else float("inf"))
    return out


# The two benchmark workloads (sphere radius 5.08 cm, ports 1.27 / 1.27 /
# 0.635 cm, wall 0.98, crosstalk on).
def bench_spheres():
    return Spheres.from_radii(5.08, 1.27, 1.27, 0.635, 0.98, R=True, T=True)


def bench0_layers():
    return [Layer.slide(1.5, 0.1), Layer(1.4, 1.0, 100.0, 0.9, 0.1), Layer.slide(1.5, 0.1)]


def bench1_layers():
    return [Layer.slide(1.52, 0.1), Layer(1.37, 0.5, 200.0, 0.8, 0.01),
            Layer(1.40, 2.0, 120.0, 0.9, 0.15), Layer(1.44, 0.2, 50.0, 0.75, 0.3),
            Layer.slide(1.52, 0.1)]
