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


# Stacks outside the golden runs' range, checked against the FP64
# restatement of the reference's walk (oracle/ismc_ref64.c):
#   anisotropy_extremes  g = -0.9, 0.99, 1 and 0; two layers index-matched to
#                        the ambient (n = 1); the benchmark spheres
#   index_contrast       n = 2.4 tissue 20 um thick under an n = 1.8 slide, a
#                        strong absorber (mua 30), a highly scattering layer
#                        (mus 300, g 0.95), an n = 1.45 slide; large ports,
#                        unequal walls and both angle thresholds
#   sphere_extremes      a thin slab between slides under a lossless R sphere
#                        (wall 1.0) with a 0.2 % sample port and a 30 %
#                        entrance port; no T sphere, with the reference's
#                        0.22-degree acceptance angle
def extreme_stacks():
    return {
        "anisotropy_extremes": (
            [Layer(1.0, 0.5, 40.0, -0.9, 0.1), Layer(1.0, 0.2, 60.0, 0.99, 0.1),
             Layer(1.33, 0.3, 30.0, 1.0, 0.05), Layer(1.33, 0.1, 20.0, 0.0, 0.05)],
            bench_spheres()),
        "index_contrast": (
            [Layer.slide(1.8, 0.05), Layer(2.4, 0.2, 80.0, 0.85, 0.002),
             Layer(1.33, 30.0, 5.0, 0.5, 0.05), Layer(1.55, 0.05, 300.0, 0.95, 0.08),
             Layer.slide(1.45, 0.2)],
            Spheres(R=True, R_pw=0.995, R_fs=0.08, R_fp=0.06, R_fd=0.02, R_angle=0.3,
                    T=True, T_pw=0.9, T_fs=0.12, T_fp=0.01, T_fd=0.05, T_angle=0.01)),
        "sphere_extremes": (
            [Layer.slide(1.5, 0.1), Layer(1.4, 0.3, 30.0, 0.8, 0.05), Layer.slide(1.5, 0.1)],
            Spheres(R=True, R_pw=1.0, R_fs=0.002, R_fp=0.3, R_fd=0.01, R_angle=0.2,
                    T=False, T_pw=0.9, T_fs=0.1, T_fp=0.1, T_fd=0.1,
                    T_angle=0.22 * math.pi / 180)),
    }


# Stacks for the physical mode (no counterpart in the reference), checked
# against the FP64 physical walk of oracle/ismc_ref64.c:
#   bench1                   the multilayer benchmark stack
#   absorbing_slides         slides that absorb (mua 0.8 and 2.0: Beer-Lambert)
#                            around the single-layer slab
#   index_contrast           the extreme index-contrast stack above
#   slab_slides_T_only       the single-layer configuration, T sphere only
def physical_stacks():
    return {
        "bench1": (bench1_layers(), bench_spheres()),
        "absorbing_slides": ([Layer(1.5, 0.8, 0.0, 0.0, 0.1), Layer(1.4, 1.0, 100.0, 0.9, 0.1),
                              Layer(1.45, 2.0, 0.0, 0.0, 0.15)], bench_spheres()),
        "index_contrast": extreme_stacks()["index_contrast"],
        "slab_slides_T_only": (bench0_layers(),
                               Spheres.from_radii(5.08, 1.27, 1.27, 0.635, 0.98, R=False, T=True)),
    }
