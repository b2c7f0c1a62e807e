"""The reference's own Python forward model as bench.py's CPU reference arm
(oracle/refpython.py over the ISMLMC.py / MLMC.py copies staged by
oracle/build_ref.py).  Skipped where nothing was staged."""
import pytest

from oracle import build_ref, refpython


def _model():
    d = build_ref.staged_python()
    if d is None:
        pytest.skip("the reference's Python model was not staged")
    return d


def test_refpython_pool_runs_the_reference_model():
    """Two workers run the reference's ISMLMC() on the multilayer benchmark
    stack: the five tallies account for every packet's weight (they sum to 1 up
    to the reference's rounding) and the run repeats exactly for the same seed."""
    from ismc_gb300 import workloads as W
    layers = refpython.layer_tuples(W.bench1_layers())
    sph = refpython.sphere_dict(W.bench_spheres())
    with refpython.Runner(_model(), 2) as pool:
        t1, wall, cpu = pool.run(layers, sph, 200, 11)
        t2, _, _ = pool.run(layers, sph, 200, 11)
    assert t1 == t2
    assert abs(sum(t1) - 1.0) < 1e-2
    assert all(0.0 <= v <= 1.0 for v in t1)
    assert wall > 0 and cpu > 0


def test_instance_args_match_the_layer_and_sphere_helpers():
    """The reference's arguments read back from a C-ABI instance equal those
    built from the Layer / Spheres objects it was made from."""
    from ismc_gb300 import make_instance
    from ismc_gb300 import workloads as W
    layers, sph = W.bench1_layers(), W.bench_spheres()
    la, sa = refpython.instance_args(make_instance(layers, sph, 1000))
    lb, sb = refpython.layer_tuples(layers), refpython.sphere_dict(sph)
    assert len(la) == len(lb)
    for a, b in zip(la, lb):
        assert a == pytest.approx(b, rel=1e-6)          # the instance stores float32
    assert set(sa) == set(sb)
    for k in sb:
        assert sa[k] == pytest.approx(float(sb[k]), rel=1e-12), k


def test_bench_refpython_arm_prints_its_line():
    """bench.py --impl reference --workload refpython: one JSON line with the
    reference arm's keys, on a tiny explicit packet count."""
    import json
    import os
    import subprocess
    import sys
    _model()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--workload", "refpython", "--stack", "bench0", "--packets", "400",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["workload"] == "refpython"
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "reference"
    assert line["config"]["packets_per_step"] >= 400
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert abs(sum(line["result"]["mean"]) - 1.0) < 0.05


def test_refpython_baseline_line():
    """The GPU arm's cpu_baseline where the reference's Python is staged: a
    bounded sample on every host core, kind "reference"."""
    import os
    import sys
    _model()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    b = bench.refpython_baseline(seconds=0.2, stack="bench0")
    assert b["kind"] == "reference" and b["value"] > 0
    assert b["cores"] == bench.host_cores() and "ISMLMC.py" in b["sample"]
