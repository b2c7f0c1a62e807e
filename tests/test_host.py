"""Host-side helpers that need no GPU: the vectorised instance builder and
tally normalisation agree with their one-at-a-time counterparts."""
import math

import numpy as np
import pytest

from ismc_gb300 import _abi, api
from ismc_gb300.surrogate import sample_stack
from ismc_gb300.workloads import bench_spheres


def test_slab_instances_are_byte_identical_to_make_instance():
    rng = np.random.default_rng(0)
    X = np.stack([rng.uniform(-4.6, 2.3, 64), rng.uniform(0, 4.6, 64), rng.uniform(0.6, 1.0, 64),
                  rng.uniform(0.02, 0.5, 64), rng.uniform(1.33, 1.5, 64)], 1)
    X[3, 2] = 1.0                                 # g = 1: mu_s = mu_s'
    sph = bench_spheres()
    for mode in ("compat", "physical"):
        arr = api.slab_instances(np.exp(X[:, 0]), np.exp(X[:, 1]), X[:, 2], X[:, 3], X[:, 4], sph,
                                 54321, seed=(1 << 40) + 7, stream0=1000, mode=mode)
        for i, r in enumerate(X):
            ref = api.make_instance(sample_stack(math.exp(r[0]), math.exp(r[1]), r[2], r[3], r[4]),
                                    sph, 54321, seed=(1 << 40) + 7, stream=1000 + i, mode=mode)
            assert bytes(arr[i]) == bytes(ref), i


def test_tallies_mean_se_matches_tally_to_result():
    rng = np.random.default_rng(1)
    out = (_abi.Tally * 6)()
    for i, t in enumerate(out):
        t.n = [0, 1, 2, 1000, 123457, 10 ** 8][i]
        t.scale_log2 = 32
        for k in range(5):
            m = float(rng.random())
            t.sum[k] = int(m * t.n * 2 ** 32)
            t.sumsq[k] = int(m * m * 1.3 * t.n * 2 ** 32)
        t.status = -3 if i == 2 else 0
    mean, se, status = api.tallies_mean_se(out)
    for i, t in enumerate(out):
        r = api.tally_to_result(t)
        assert status[i] == r.status
        for k in range(5):
            if math.isnan(r.mean[k]):
                assert np.isnan(mean[i, k]) and np.isnan(se[i, k])
            else:
                assert mean[i, k] == r.mean[k] and se[i, k] == r.se[k], (i, k)


def _grid_loop(mu_a, musr, g, t, n, spheres, N, runs, separate, seed, stream0, slides, mode):
    """The one-instance-at-a-time construction the vectorised grid builder replaces."""
    from ismc_gb300 import Layer, Spheres
    mus = np.asarray(musr, float) / (1 - g) if g != 1 else np.asarray(musr, float)
    thr = 1e-3 if slides is None else 1e-4
    sp_R = Spheres(**{**spheres.__dict__, "T": False})
    sp_T = Spheres(**{**spheres.__dict__, "R": False})
    out, stream = [], stream0
    for a in np.asarray(mu_a, float):
        for s in mus:
            tissue = Layer(n, float(a), float(s), g, t)
            layers = [tissue] if slides is None else [slides[0], tissue, slides[1]]
            for _ in range(runs):
                for sp in ((sp_R, sp_T) if separate else (spheres,)):
                    out.append(api.make_instance(layers, sp, N, seed=seed, stream=stream, mode=mode,
                                                 roulette_threshold=thr))
                    stream += 1
    return out


def test_grid_instances_are_byte_identical_to_the_loop():
    from ismc_gb300 import Layer
    from ismc_gb300.lookup import _grid_instances
    mu_a = 0.5 * 1.2 ** np.arange(5)
    musr = 10 * 1.3 ** np.arange(4)
    sph = bench_spheres()
    for slides in (None, (Layer.slide(1.5, 0.1), Layer.slide(1.52, 0.12))):
        for separate, runs in ((True, 2), (False, 3)):
            arr, index = _grid_instances(mu_a, musr, 0.9, 0.135, 1.41, sph, 7777, runs, separate,
                                         12, 500, slides, "compat")
            ref = _grid_loop(mu_a, musr, 0.9, 0.135, 1.41, sph, 7777, runs, separate, 12, 500,
                             slides, "compat")
            assert len(arr) == len(ref)
            for a, b in zip(arr, ref):
                assert bytes(a) == bytes(b)
            assert index["i"].max() == 4 and index["j"].max() == 3 and index["r"].max() == runs - 1


def test_component_costs_from_an_ncu_csv(tmp_path):
    """ismc_gb300.perf turns an ncu CSV of the building-block kernels into
    warp instructions per call, with the shared loop's overhead subtracted."""
    from ismc_gb300 import perf
    warps_calls = perf._WARPS * perf._ITERS
    hdr = ('"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream",'
           '"Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit",'
           '"Metric Value"')

    def row(i, k, m, v):
        return (f'"{i}","1","components","h","{k}(float *, unsigned int)","1","7","(256, 1, 1)",'
                f'"(608, 1, 1)","0","10.3","Command line profiler metrics","{m}","inst","{v}"')
    lines = ["==PROF== Connected", hdr,
             row(0, "k_loop", "smsp__inst_executed.sum", int(3.25 * warps_calls)),
             row(0, "k_loop", "smsp__thread_inst_executed.sum", int(3.25 * warps_calls * 32)),
             row(1, "k_div", "smsp__inst_executed.sum", int(16.25 * warps_calls)),
             row(1, "k_div", "smsp__thread_inst_executed.sum", int(16.25 * warps_calls * 30))]
    p = tmp_path / "c.csv"
    p.write_text("\n".join(lines) + "\n")
    got = perf.components_from_csv(str(p))
    assert abs(got["div"]["warp_inst_per_call"] - 13.0) < 1e-9
    assert abs(got["div"]["lanes"] - 30.0) < 1e-9
    assert abs(got["_loop_overhead"] - 3.25) < 1e-9


def test_reference_cuda_arm_refuses_stacks_with_slides(capsys):
    """The reference kernel is timed only on slide-less stacks: on a stack with
    slides the arm prints its unavailable line and runs nothing."""
    import argparse
    import json
    import bench
    bench.run_refcuda(argparse.Namespace(stack="bench1", packets=10**8, steps=1, warmup=1), 0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["workload"] == "refcuda"
    assert "slides" in line["unavailable"]


def test_split_instance_covers_the_packet_range_once():
    """An instance above the per-instance packet limit becomes consecutive
    packet ranges of the same simulation."""
    from ismc_gb300 import Layer, Spheres, make_instance, split_instance
    inst = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], Spheres(), 10_500_000, seed=3,
                         packet_offset=7)
    assert split_instance(inst) == [inst]
    parts = split_instance(inst, max_packets=4_000_000)
    assert [(int(p.packet_offset), int(p.n_packets)) for p in parts] == \
        [(7, 4_000_000), (4_000_007, 4_000_000), (8_000_007, 2_500_000)]
    for p in parts:
        assert bytes(p.stack) == bytes(inst.stack) and int(p.seed) == 3


def test_merge_tallies_adds_exactly_beyond_64_bits():
    """Merged tallies keep exact integer sums (past 2^64) and normalise like a
    single tally."""
    from ismc_gb300 import _abi, merge_tallies, tally_to_result
    a, b = _abi.Tally(), _abi.Tally()
    for t, n, w in ((a, 1000, 0.25), (b, 3000, 0.75)):
        t.n = n
        t.scale_log2 = 32
        t.sum[1] = int(n * w * 2 ** 32)
        t.sumsq[1] = int(n * w * w * 2 ** 32)
        t.steps = n * 10
    m = merge_tallies([a, b])
    assert m.n == 4000 and m.steps == 40000
    assert m.mean[1] == pytest.approx((250 + 2250) / 4000, rel=1e-15)
    one = tally_to_result(a)
    assert one.mean[1] == pytest.approx(0.25, rel=1e-15) and one.se[1] == 0.0
    big = [_abi.Tally() for _ in range(3)]
    for t in big:
        t.n = 2 ** 31
        t.scale_log2 = 32
        t.sum[0] = 2 ** 63                      # weight 1 per packet at 2^32
        t.sumsq[0] = 2 ** 63
    r = merge_tallies(big)
    assert r.sums[0] == 3 * 2 ** 63 and r.mean[0] == 1.0 and r.se[0] == 0.0


def test_bench_clock_sampler_against_a_fake_nvidia_smi(tmp_path, monkeypatch):
    """bench.py's clock record: median SM clock under load, the maximum, and
    the throttle reasons that were active, from nvidia-smi's CSV rows (a
    stand-in script here); entering the sampler waits for its first row."""
    import os
    import stat
    import sys
    fake = tmp_path / "nvidia-smi"
    rows = ["0, 2070, 2070, 800.5, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 2070, 2070, 900.1, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 1965, 2070, 1000.0, 0x4, Not Active, Not Active, Not Active, Active"]
    fake.write_text("#!/bin/sh\nsleep 0.3\n" + "".join(f"echo '{r}'\n" for r in rows) +
                    "sleep 5\n")
    fake.chmod(fake.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ["PATH"])
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    with bench.ClockSampler(0) as clk:
        assert clk.rows                      # the first sample is in before timing starts
        import time
        time.sleep(0.3)
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3
