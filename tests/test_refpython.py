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
