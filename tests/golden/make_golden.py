"""Generate the statistical golden fixtures from the reference's own Python.

This script runs ONLY where the reference checkout is available (it imports
the reference's ``ISMC.py`` / ``ISMLMC.py`` / ``MLMC.py`` read-only through
``sys.path``).  The GPU machine never runs it: the fixtures it writes
(``tests/golden/reference_cases.json``) are committed and travel instead.

Each case is run as K independent batches under ``multiprocessing`` (spawn
start method), batch k seeded with ``random.seed(base_seed + k)``.  The batch
means give the reference estimate, and their spread gives a batch-mean
standard error that does not rely on the Poisson approximation the reference
prints (ISMC.py:419-432).

Usage:  python tests/golden/make_golden.py /path/to/reference [--only NAME]
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_cases.json")

# Two-sphere geometry of the benchmark workloads: spheres of radius 5.08 cm,
# sample and entrance ports of radius 1.27 cm, detector port 0.635 cm,
# wall reflectance 0.98.  The reference takes port AREA fractions
# (Lookup/example.ini:21-31); a circular port of radius a on a sphere of
# radius Rs covers the spherical cap fraction f = (1 - sqrt(1 - (a/Rs)^2))/2.
def cap_fraction(a, Rs=5.08):
    return 0.5 * (1.0 - math.sqrt(1.0 - (a / Rs) ** 2))


FS = cap_fraction(1.27)
FP = cap_fraction(1.27)
FD = cap_fraction(0.635)
PW = 0.98

BENCH_SPHERES = dict(R=True, R_pw=PW, R_fs=FS, R_fp=FP, R_fd=FD, R_f=FS + FP + FD,
                     R_angle=math.pi / 10, specular_included=False,
                     T=True, T_pw=PW, T_fs=FS, T_fp=FP, T_fd=FD, T_f=FS + FP + FD,
                     T_angle=0.22 * math.pi / 180)


def spheres(**over):
    d = dict(BENCH_SPHERES)
    d.update(over)
    return d


def layer(n, mua, mus, g, d):
    return dict(n=n, mua=mua, mus=mus, g=g, d=d)


GLASS15 = layer(1.5, 0.0, 0.0, 0.0, 0.1)
GLASS152 = layer(1.52, 0.0, 0.0, 0.0, 0.1)
SLAB0 = layer(1.4, 1.0, 100.0, 0.9, 0.1)

# name -> (driver, layers, spheres, N, K, base_seed).  64 batches per case, so
# that the batch-mean standard error is itself known to ~9 % and the 3-sigma
# comparison of tests/test_gpu_parity.py holds for a correct implementation
# with the normal tail probability (0.27 % per tally).
#   driver "ISMLMC": ISMLMC.ISMLMC (multilayer, roulette threshold 1e-4)
#   driver "ISMC":   ISMC.ISMC     (single slab, roulette threshold 1e-3)
CASES = {
    # benchmark workload 0: slab between two n=1.5 slides, both spheres, crosstalk
    "bench0_slides": ("ISMLMC", [GLASS15, SLAB0, GLASS15], spheres(), 400000, 64, 1000),
    # benchmark workload 1: three tissue layers between n=1.52 slides
    "bench1_multilayer": ("ISMLMC", [GLASS152,
                                     layer(1.37, 0.5, 200.0, 0.8, 0.01),
                                     layer(1.40, 2.0, 120.0, 0.9, 0.15),
                                     layer(1.44, 0.2, 50.0, 0.75, 0.3),
                                     GLASS152], spheres(), 4000000, 64, 2000),
    # workload 0 without slides, single-slab driver, every sphere combination
    "slab_both": ("ISMC", [SLAB0], spheres(), 400000, 64, 3000),
    "slab_R_only": ("ISMC", [SLAB0], spheres(T=False), 400000, 64, 3100),
    "slab_T_only": ("ISMC", [SLAB0], spheres(R=False), 400000, 64, 3200),
    "slab_no_spheres": ("ISMC", [SLAB0], spheres(R=False, T=False), 400000, 64, 3300),
    "slab_specular_included": ("ISMC", [SLAB0], spheres(specular_included=True), 400000, 64, 3400),
    # the single-slab example of ISMC.py:19-50 (R sphere only)
    "ismc_example": ("ISMC", [layer(1.4, 1.78, 31.2 / 0.5, 0.5, 0.135)],
                     dict(R=True, R_pw=0.99, R_fs=0.02351, R_fp=0.054638, R_fd=0.02351,
                          R_f=0.02351 + 0.054638 + 0.02351, R_angle=math.pi / 10,
                          specular_included=False, T=False, T_pw=0.99, T_fs=0.054638,
                          T_fp=0.02351, T_fd=0.02351, T_f=0.054638 + 0.02351 + 0.02351,
                          T_angle=0.22 * math.pi / 180), 400000, 64, 3500),
    # the three-layer example of ISMLMC.py:20-55 (isotropic middle layer, no spheres)
    "ismlmc_example": ("ISMLMC", [layer(1.37, 1.0, 10.0 / 0.1, 0.9, 0.1),
                                  layer(1.37, 1.0, 10.0, 0.0, 0.1),
                                  layer(1.37, 2.0, 3.0 / 0.3, 0.7, 0.2)],
                       dict(R=False, R_pw=0.85, R_fs=0.1, R_fp=0.05, R_fd=0.05, R_f=0.2,
                            R_angle=math.pi / 10, specular_included=False,
                            T=False, T_pw=0.85, T_fs=0.1, T_fp=0.05, T_fd=0.05, T_f=0.2,
                            T_angle=math.pi / 10), 400000, 64, 3600),
    # lookup-grid corners (single slab between n=1.5 slides, n=1.4, g=0.9)
    "grid_low_albedo_thin": ("ISMLMC", [GLASS15, layer(1.4, 10.0, 1.0 / 0.1, 0.9, 0.05), GLASS15],
                             spheres(), 400000, 64, 3700),
    "grid_high_albedo_thick": ("ISMLMC", [GLASS15, layer(1.4, 0.01, 100.0 / 0.1, 0.9, 0.2), GLASS15],
                               spheres(), 80000, 64, 3800),
    # five tissue layers with distinct indices, slides n=1.5, mixed anisotropy
    "five_layer_mixed": ("ISMLMC", [GLASS15,
                                    layer(1.33, 0.3, 80.0, 0.8, 0.05),
                                    layer(1.45, 3.0, 40.0, 0.6, 0.08),
                                    layer(1.38, 0.05, 150.0, 0.95, 0.1),
                                    layer(1.50, 1.0, 20.0, 0.0, 0.03),
                                    layer(1.36, 0.5, 60.0, 0.9, 0.12),
                                    GLASS15], spheres(), 200000, 64, 3900),
    # the multilayer benchmark stack with the 8-degree launch (specular_included):
    # the tilted launch through the slide's two-interface series
    "bench1_specular_included": ("ISMLMC", [GLASS152,
                                            layer(1.37, 0.5, 200.0, 0.8, 0.01),
                                            layer(1.40, 2.0, 120.0, 0.9, 0.15),
                                            layer(1.44, 0.2, 50.0, 0.75, 0.3),
                                            GLASS152], spheres(specular_included=True),
                                 400000, 64, 4100),
    # the single-layer benchmark stack with no spheres: acceptance by angle
    # (ISMLMC.py:163, 211, 273, 325) behind slides
    "bench0_no_spheres": ("ISMLMC", [GLASS15, SLAB0, GLASS15], spheres(R=False, T=False),
                          400000, 64, 4200),
    # tissue directly against ambient on both faces, both spheres, thicker slab
    "bare_two_layer": ("ISMLMC", [layer(1.4, 0.5, 50.0, 0.85, 0.1),
                                  layer(1.33, 0.2, 30.0, 0.7, 0.2)], spheres(), 400000, 64, 4000),
    # anisotropy extremes: back-scattering, strongly forward, undeflected and
    # isotropic layers, the first two index-matched to the ambient (n = 1)
    "anisotropy_extremes": ("ISMLMC", [layer(1.0, 0.5, 40.0, -0.9, 0.1),
                                       layer(1.0, 0.2, 60.0, 0.99, 0.1),
                                       layer(1.33, 0.3, 30.0, 1.0, 0.05),
                                       layer(1.33, 0.1, 20.0, 0.0, 0.05)], spheres(),
                            2000000, 64, 4300),
    # strong index contrast: n = 2.4 tissue 20 um thick under an n = 1.8 slide,
    # a strong absorber, a highly scattering layer, an n = 1.45 slide; large
    # ports, unequal walls, both angle thresholds
    "index_contrast": ("ISMLMC", [layer(1.8, 0.0, 0.0, 0.0, 0.05),
                                  layer(2.4, 0.2, 80.0, 0.85, 0.002),
                                  layer(1.33, 30.0, 5.0, 0.5, 0.05),
                                  layer(1.55, 0.05, 300.0, 0.95, 0.08),
                                  layer(1.45, 0.0, 0.0, 0.0, 0.2)],
                       dict(R=True, R_pw=0.995, R_fs=0.08, R_fp=0.06, R_fd=0.02,
                            R_f=0.08 + 0.06 + 0.02, R_angle=0.3, specular_included=False,
                            T=True, T_pw=0.9, T_fs=0.12, T_fp=0.01, T_fd=0.05,
                            T_f=0.12 + 0.01 + 0.05, T_angle=0.01), 2000000, 64, 4400),
    # sphere extremes: a lossless R sphere with a 0.2 % sample port and a 30 %
    # entrance port; no T sphere, the reference's 0.22-degree acceptance angle
    "sphere_extremes": ("ISMLMC", [GLASS15, layer(1.4, 0.3, 30.0, 0.8, 0.05), GLASS15],
                        dict(R=True, R_pw=1.0, R_fs=0.002, R_fp=0.3, R_fd=0.01,
                             R_f=0.002 + 0.3 + 0.01, R_angle=0.2, specular_included=False,
                             T=False, T_pw=0.9, T_fs=0.1, T_fp=0.1, T_fd=0.1,
                             T_f=0.1 + 0.1 + 0.1, T_angle=0.22 * math.pi / 180), 2000000, 64,
                        4500),
    # a non-absorbing thin layer between slides: no roulette, weight 1 to the end
    "nonabsorbing_thin": ("ISMLMC", [GLASS15, layer(1.4, 0.0, 50.0, 0.9, 0.02), GLASS15],
                          spheres(), 2000000, 64, 4600),
    # single-slab driver with the 8-degree launch, T sphere only (R by angle)
    "slab_specular_T_only": ("ISMC", [layer(1.33, 0.5, 20.0, 0.8, 0.2)],
                             spheres(R=False, specular_included=True), 2000000, 64, 4700),
    # three isotropic layers of different index, no slides, both spheres
    "isotropic_stack": ("ISMLMC", [layer(1.3, 0.1, 10.0, 0.0, 0.1),
                                   layer(1.5, 0.3, 25.0, 0.0, 0.05),
                                   layer(1.4, 0.05, 15.0, 0.0, 0.15)], spheres(),
                        2000000, 64, 4800),
}


def _run_batch(args):
    ref_dir, driver, layers, sph, n, seed = args
    sys.path.insert(0, ref_dir)
    import random
    random.seed(seed)
    nl = [L["n"] for L in layers]
    g = [L["g"] for L in layers]
    t = [L["d"] for L in layers]
    mua = [L["mua"] for L in layers]
    mus = [L["mus"] for L in layers]
    mut = [a + s for a, s in zip(mua, mus)]
    s = sph
    common = (s["R"], s["R_pw"], s["R_fs"], s["R_fp"], s["R_fd"], s["R_f"], s["R_angle"],
              s["specular_included"], s["T"], s["T_pw"], s["T_fs"], s["T_fp"], s["T_fd"],
              s["T_f"], s["T_angle"])
    t0 = time.time()
    if driver == "ISMC":
        import ISMC
        assert len(layers) == 1
        out = ISMC.ISMC(n, nl[0], g[0], t[0], mua[0], mus[0], mut[0], *common)
    else:
        import ISMLMC
        out = ISMLMC.ISMLMC(n, nl, g, t, mua, mus, mut, *common)
    return list(out), time.time() - t0


def run_case(pool, ref_dir, name, spec):
    driver, layers, sph, N, K, base = spec
    per = N // K
    jobs = [(ref_dir, driver, layers, sph, per, base + k) for k in range(K)]
    t0 = time.time()
    res = pool.map(_run_batch, jobs)
    wall = time.time() - t0
    batches = [r[0] for r in res]
    cpu = sum(r[1] for r in res)
    mean = [sum(b[i] for b in batches) / K for i in range(5)]
    se = [math.sqrt(sum((b[i] - mean[i]) ** 2 for b in batches) / (K - 1) / K) for i in range(5)]
    return dict(driver=driver, layers=layers, spheres=sph, packets_per_batch=per, batches=K,
                base_seed=base, tallies=["A", "R_d", "R_s", "T_d", "T_u"], batch_values=batches,
                mean=mean, se=se, cpu_seconds=cpu, wall_seconds=wall,
                packets_per_cpu_second=per * K / cpu)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference_dir")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    a = ap.parse_args()
    ref_dir = os.path.abspath(a.reference_dir)
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as fh:
            data = json.load(fh).get("cases", {})
    ctx = mp.get_context("spawn")
    with ctx.Pool(a.procs) as pool:
        for name, spec in CASES.items():
            if a.only and name not in a.only:
                continue
            r = run_case(pool, ref_dir, name, spec)
            data[name] = r
            print(f"{name}: mean={['%.5f' % m for m in r['mean']]} se={['%.1e' % s for s in r['se']]} "
                  f"wall={r['wall_seconds']:.1f}s rate={r['packets_per_cpu_second']:.0f}/s/core", flush=True)
            with open(OUT, "w") as fh:
                json.dump({"generator": "tests/golden/make_golden.py",
                           "reference": "pdcook/ISMC ISMC.py / ISMLMC.py / MLMC.py",
                           "cases": data}, fh, indent=1)


if __name__ == "__main__":
    main()
