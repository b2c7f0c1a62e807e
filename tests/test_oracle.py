"""CPU tests of the oracles against the reference's golden vectors.

Statistical rule (applies to every tally A, R_d, R_s, T_d, T_u):
    |x_a - x_b| <= Z * sqrt(se_a^2 + se_b^2)
Z = 3 for the two benchmark workloads (the parity bar: 3 combined standard
errors).  The other golden cases are checked as one family with a Bonferroni
bound so that the family-wise false-alarm rate stays at the 3-sigma level
(0.27 %): Z = 4.0 for up to 60 comparisons.
"""
import math

import numpy as np
import pytest

import cases
import oracle
from ismc_gb300 import tally_to_result

HEADLINE = ("bench0_slides", "bench1_multilayer")
Z_HEADLINE = 3.0
Z_FAMILY = 4.0
# packets per oracle run (the oracles are C: these take well under a second each)
ORACLE_N = {"bench1_multilayer": 1_000_000, "grid_high_albedo_thick": 100_000}


def _z(case_name, case, mean, se):
    z = cases.zscores(mean, se, case["mean"], case["se"])
    lim = Z_HEADLINE if case_name in HEADLINE else Z_FAMILY
    return z, lim


@pytest.mark.parametrize("name", sorted(cases.golden()))
def test_twin_matches_reference(name):
    c = cases.golden()[name]
    n = ORACLE_N.get(name, 400_000)
    r = tally_to_result(oracle.twin_run(cases.case_instance(c, n, seed=20240601)))
    z, lim = _z(name, c, r.mean, r.se)
    assert max(abs(x) for x in z) <= lim, f"{name}: z={z}"


@pytest.mark.parametrize("name", sorted(cases.golden()))
def test_ref64_matches_reference(name):
    c = cases.golden()[name]
    n = ORACLE_N.get(name, 400_000)
    mean, se, _ = oracle.ref64_run(cases.case_instance(c, n, seed=99), single=c["driver"] == "ISMC")
    z, lim = _z(name, c, mean, se)
    assert max(abs(x) for x in z) <= lim, f"{name}: z={z}"


def test_twin_vs_ref64_large_n():
    """The FP32 event restatement and the FP64 structural restatement agree at
    2e6 packets (standard errors ~3e-4)."""
    c = cases.golden()["bench0_slides"]
    inst = cases.case_instance(c, 2_000_000, seed=5)
    r = tally_to_result(oracle.twin_run(inst))
    mean, se, _ = oracle.ref64_run(inst)
    z = cases.zscores(r.mean, r.se, mean, se)
    assert max(abs(x) for x in z) <= Z_FAMILY, z


@pytest.mark.parametrize("name", sorted(cases.extreme_stacks()))
def test_twin_vs_ref64_extreme_stacks(name):
    """The FP32 twin's division-free Henyey-Greenstein, rotation and Fresnel
    algebra against the FP64 restatement of the reference's walk on stacks
    the golden runs do not reach (tests/cases.py extreme_stacks), 3 combined
    standard errors per tally.  The GPU draws the twin's tallies bit for
    bit, so its test of the same stacks sees the same z-scores."""
    layers, sph = cases.extreme_stacks()[name]
    from ismc_gb300 import make_instance
    r = tally_to_result(oracle.twin_run(make_instance(layers, sph, 2_000_000, seed=22)))
    mean, se, _ = oracle.ref64_run(make_instance(layers, sph, 400_000, seed=23))
    z = cases.zscores(r.mean, r.se, mean, se)
    assert max(abs(x) for x in z) <= 3.0, z


@pytest.mark.parametrize("name", sorted(cases.physical_stacks()))
def test_twin_vs_ref64_physical_mode(name):
    """The physical mode (optical depth kept across slides, Beer-Lambert in
    slides, one Fresnel draw at incidence, cosine-weighted re-incidence) of
    the FP32 twin against the independent FP64 physical walk of
    oracle/ismc_ref64.c, 3 combined standard errors per tally.  The GPU draws
    the twin's tallies bit for bit."""
    from ismc_gb300 import make_instance
    layers, sph = cases.physical_stacks()[name]
    r = tally_to_result(oracle.twin_run(make_instance(layers, sph, 2_000_000, seed=22,
                                                      mode="physical")))
    mean, se, _ = oracle.ref64_run(make_instance(layers, sph, 1_000_000, seed=23,
                                                 mode="physical"))
    z = cases.zscores(r.mean, r.se, mean, se)
    assert max(abs(x) for x in z) <= 3.0, z


def test_twin_thread_invariance():
    """Integer tallies do not depend on how packets are split across threads."""
    c = cases.golden()["five_layer_mixed"]
    inst = cases.case_instance(c, 20_000, seed=3)
    a, b = oracle.twin_run(inst, threads=1), oracle.twin_run(inst, threads=7)
    assert list(a.sum) == list(b.sum) and list(a.sumsq) == list(b.sumsq)
    assert a.steps == b.steps and a.events == b.events


def test_twin_sharding_is_exact():
    """Packet ranges [0,k) + [k,n) sum to the tallies of [0,n) bit for bit."""
    c = cases.golden()["bench0_slides"]
    whole = oracle.twin_run(cases.case_instance(c, 30_000, seed=11))
    p1 = oracle.twin_run(cases.case_instance(c, 12_345, seed=11))
    p2 = oracle.twin_run(cases.case_instance(c, 30_000 - 12_345, seed=11, packet_offset=12_345))
    for k in range(5):
        assert whole.sum[k] == p1.sum[k] + p2.sum[k]
        assert whole.sumsq[k] == p1.sumsq[k] + p2.sumsq[k]


def test_weight_conservation():
    """Every launched unit of weight ends in exactly one tally, up to roulette
    (unbiased) and fixed-point rounding."""
    c = cases.golden()["bench1_multilayer"]
    r = tally_to_result(oracle.twin_run(cases.case_instance(c, 200_000, seed=8)))
    tot = sum(r.mean)
    se = math.sqrt(sum(s * s for s in r.se))
    assert abs(tot - 1.0) < 5 * se + 1e-6, (tot, se)


# ----------------------------------------------------------------------------
# RNG and elementary functions
# ----------------------------------------------------------------------------
def _philox(ctr, key, W, M, Wc, rounds=10):
    mask = (1 << W) - 1
    c, k = list(ctr), list(key)
    for r in range(rounds):
        if r:
            k = [(k[0] + Wc[0]) & mask, (k[1] + Wc[1]) & mask]
        p0, p1 = M[0] * c[0], M[1] * c[2]
        c = [(p1 >> W) ^ c[1] ^ k[0], p1 & mask, (p0 >> W) ^ c[3] ^ k[1], p0 & mask]
    return c


def test_philox_round_structure_matches_numpy_4x64():
    """The round function / key schedule, instantiated at 64-bit width with the
    published 4x64 constants, reproduces numpy's independent Philox4x64-10
    (numpy increments its counter before each block)."""
    M = (0xD2E7470EE14C6C93, 0xCA5A826395121157)
    Wc = (0x9E3779B97F4A7C15, 0xBB67AE8584CAA73B)
    key = [0x0123456789ABCDEF, 0xFEDCBA9876543210]
    for start in (0, 5, 2**40):
        bg = np.random.Philox(key=np.array(key, dtype=np.uint64),
                              counter=np.array([start, 0, 0, 0], dtype=np.uint64))
        raw = [int(x) for x in bg.random_raw(4)]
        assert raw == _philox([start + 1, 0, 0, 0], key, 64, M, Wc)


def test_philox_4x32_twin_matches_python():
    import ctypes as C
    M = (0xD2511F53, 0xCD9E8D57)
    Wc = (0x9E3779B9, 0xBB67AE85)
    rng = np.random.default_rng(1)
    for _ in range(200):
        ctr = [int(x) for x in rng.integers(0, 2**32, 4)]
        key = [int(x) for x in rng.integers(0, 2**32, 2)]
        out = (C.c_uint32 * 4)()
        oracle.lib().twin_philox((C.c_uint32 * 4)(*ctr), key[0], key[1], out)
        assert list(out) == _philox(ctr, key, 32, M, Wc)


def test_philox_4x32_uniformity_and_independence():
    """Chi-square uniformity of each output word's top byte and lag-1 correlation
    across consecutive counters are at noise level."""
    import ctypes as C
    L = oracle.lib()
    n = 40000
    words = np.empty((n, 4), dtype=np.uint64)
    out = (C.c_uint32 * 4)()
    for i in range(n):
        L.twin_philox((C.c_uint32 * 4)(i, 7, 0, 3), 0xABCDEF01, 0x12345678, out)
        words[i] = list(out)
    u = words / 2.0**32
    for j in range(4):
        h = np.bincount((words[:, j] >> 24).astype(np.int64), minlength=256)
        chi2 = ((h - n / 256) ** 2 / (n / 256)).sum()
        assert chi2 < 255 + 6 * math.sqrt(2 * 255), chi2
        corr = np.corrcoef(u[:-1, j], u[1:, j])[0, 1]
        assert abs(corr) < 5 / math.sqrt(n), corr
    cross = np.corrcoef(u.T)
    assert np.max(np.abs(cross - np.eye(4))) < 5 / math.sqrt(n)


def test_uniform_open_interval():
    L = oracle.lib()
    assert 0.0 < L.twin_u01(0) < 1e-6
    assert 1.0 - 1e-6 < L.twin_u01(0xFFFFFFFF) < 1.0


def test_neglog_accuracy():
    L = oracle.lib()
    xs = np.unique(np.concatenate([np.arange(0, 2**32, 2**32 // 50000, dtype=np.uint64),
                                   np.arange(0, 5000, dtype=np.uint64),
                                   2**32 - 1 - np.arange(0, 5000, dtype=np.uint64)]))
    worst = 0.0
    for x in xs:
        x = int(x)
        u = np.float32(np.float32(x | 1) * np.float32(2.0 ** -32))
        ref = -math.log(float(u))
        got = L.twin_neglog_u32(x)
        if ref > 0:
            worst = max(worst, abs(got - ref) / ref)
        else:
            assert got == 0.0
    assert worst < 4e-7, worst


def test_sincos_accuracy():
    import ctypes as C
    L = oracle.lib()
    s, c = C.c_float(), C.c_float()
    worst = 0.0
    for k in range(0, 2**23, 97):
        u = float(L.twin_u01(k << 9))
        L.twin_sincos_2pi(u, C.byref(s), C.byref(c))
        worst = max(worst, abs(s.value - math.sin(2 * math.pi * u)),
                    abs(c.value - math.cos(2 * math.pi * u)))
    assert worst < 3e-7, worst


def test_expneg_accuracy():
    L = oracle.lib()
    worst = 0.0
    for x in np.linspace(0, 80, 20001, dtype=np.float32):
        ref = math.exp(-float(x))
        worst = max(worst, abs(L.twin_expneg(float(x)) - ref) / ref)
    assert worst < 4e-7, worst
    assert L.twin_expneg(100.0) == 0.0


def test_fresnel_algebraic_equals_trigonometric():
    """Algebraic Fresnel form vs the reference's trigonometric form (MLMC.py:45-54)."""
    import ctypes as C
    L = oracle.lib()
    ct = C.c_float()

    def trig(ni, nt, mz):
        if abs(mz) > 0.99999:
            return ((nt - ni) / (nt + ni)) ** 2
        ti = math.acos(abs(mz))
        if ni * math.sin(ti) / nt >= 1:
            return 1.0
        tt = math.asin(ni * math.sin(ti) / nt)
        return 0.5 * (math.sin(ti - tt) ** 2 / math.sin(ti + tt) ** 2 +
                      math.tan(ti - tt) ** 2 / math.tan(ti + tt) ** 2)

    for ni, nt in ((1.0, 1.4), (1.4, 1.0), (1.5, 1.4), (1.37, 1.52), (1.52, 1.0)):
        eta = np.float32(ni / nt)
        for mz in np.linspace(0.001, 1.0, 3001):
            got = L.twin_fresnel(float(eta), float(np.float32(mz)), C.byref(ct))
            ref = trig(ni, nt, float(np.float32(mz)))
            assert abs(got - ref) < 2e-5, (ni, nt, mz, got, ref)


def test_twin_interface_draw_without_division_matches_u_below_R():
    """The interface draw u * den^2 < (x^2 + y^2)/2 (no division) decides as
    u < R does, except where u lies within rounding of R; and it hands back
    the same refracted cosine."""
    import ctypes as C
    L = oracle.lib()
    ct, ct2 = C.c_float(), C.c_float()
    rng = np.random.default_rng(12)
    mism = 0
    for ni, nt in ((1.0, 1.4), (1.4, 1.0), (1.37, 1.52), (1.52, 1.0), (1.44, 1.52)):
        eta = float(np.float32(ni / nt))
        ci = rng.uniform(1e-4, 1.0, 4000).astype(np.float32)
        for c in ci:
            R = L.twin_fresnel(eta, float(c), C.byref(ct))
            # u on both sides of R, and right next to it
            for u in (R * 0.5, R * (1 - 1e-6), R * (1 + 1e-6), min(0.99999994, R + (1 - R) * 0.5)):
                u = float(np.float32(u))
                if not 0.0 < u < 1.0:
                    continue
                got = bool(L.twin_fresnel_reflects(eta, float(c), u, C.byref(ct2)))
                assert ct2.value == ct.value
                if got != (u < R):
                    mism += 1
                    assert abs(u - R) <= 4e-7 * max(R, 1e-30), (ni, nt, c, u, R)
    assert mism <= 20, mism


# ----------------------------------------------------------------------------
# FP64 analytic oracle
# ----------------------------------------------------------------------------
def test_analytic64_closed_forms():
    # single non-absorbing slab in air: T = (1 - r)/(1 + r), R = 2r/(1 + r)
    n = 1.5
    r = ((n - 1) / (n + 1)) ** 2
    spec, ball = oracle.analytic64([n], [0.0], [0.0], [1.0], mode="physical")
    assert abs(ball - (1 - r) / (1 + r)) < 1e-12
    assert abs(spec - 2 * r / (1 + r)) < 1e-12
    # compatible specular of a slide on tissue = the series of ISMLMC.py:89
    spec, _ = oracle.analytic64([1.5, 1.4, 1.5], [0.0, 100.0, 0.0], [0.0, 101.0, 0.0],
                                [0.1, 0.1, 0.1], mode="compat")
    a, b = float(np.float32(1.5)), float(np.float32(1.4))
    r1, r2 = ((1 - a) / (1 + a)) ** 2, ((a - b) / (a + b)) ** 2
    assert abs(spec - (r1 + (1 - r1) ** 2 * r2 / (1 - r1 * r2))) < 1e-12
    # attenuating slab: T = (1-r)^2 a / (1 - r^2 a^2)
    mu, d = 2.0, 0.3
    a = math.exp(-float(np.float32(mu)) * float(np.float32(d)))
    _, ball = oracle.analytic64([n], [0.0], [mu], [d], mode="physical")
    assert abs(ball - (1 - r) ** 2 * a / (1 - r * r * a * a)) < 1e-12


def test_cubic_table_oracle_matches_scipy_griddata():
    """Pin of the Clough-Tocher restatement: scipy.interpolate.griddata(cubic),
    the interpolation lookup.py:339-342 uses, on scattered data."""
    import numpy as np
    from scipy.interpolate import griddata
    from oracle import table64
    rng = np.random.default_rng(3)
    R = rng.random(150) * 60 + 10
    T = rng.random(150) * 40 + 5
    v = np.exp(-R / 30) * (1 + T / 50)
    N = 60
    tab = table64.cubic_table(R, T, v, N)
    g = np.linspace(0, 100, N)
    X, Y = np.meshgrid(g, g, indexing="ij")
    ref = griddata(np.stack([R, T], 1), v, (X, Y), method="cubic")
    assert np.array_equal(np.isnan(ref), np.isnan(tab))
    f = np.isfinite(ref)
    assert f.sum() > 500
    assert np.max(np.abs(ref[f] - tab[f])) < 1e-12
