"""Size-independent properties at the benchmark workloads' full sizes.

* The multilayer benchmark step, 1e8 packets of the 3-layer stack between
  n = 1.52 slides (seed 7). The same packets, split into three shards run as
  one batch, give bit-identical integer tallies and counters. The full-size
  means agree with the reference's own runs (1e6 packets, tests/golden)
  within 3 combined standard errors.
* The lookup workload at its full instance count: the 64 x 64 single-slab
  grid plus 512 random stacks, 4608 instances in one batched launch, with
  the photon budgets scaled by 1e-2 to keep the test short. For a seeded
  sample of instances, each instance's tallies from the batch equal those
  of the same instance run alone.
* 5e9 packets of the multilayer stack in one call, above the per-instance
  limit: run as consecutive packet ranges and merged exactly.
"""
import numpy as np
import pytest

import cases
from ismc_gb300 import tally_to_result

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from ismc_gb300 import Engine, build
    build.build()
    e = Engine(0)
    yield e
    e.close()


def _same(a, b):
    return (list(a.sum) == list(b.sum) and list(a.sumsq) == list(b.sumsq) and a.steps == b.steps
            and a.events == b.events and a.reincidences == b.reincidences and a.capped == b.capped
            and a.trapped == b.trapped and a.n == b.n and a.status == b.status)


def test_multilayer_benchmark_step_full_size(engine):
    c = cases.golden()["bench1_multilayer"]
    N = 100_000_000
    whole = engine.run_batch_raw([cases.case_instance(c, N, seed=7)])[0]
    assert whole.status == 0 and whole.n == N
    cuts = [0, 31_415_926, 77_777_777, N]
    parts = engine.run_batch_raw([cases.case_instance(c, b - a, seed=7, packet_offset=a)
                                  for a, b in zip(cuts[:-1], cuts[1:])])
    for k in range(5):
        assert whole.sum[k] == sum(p.sum[k] for p in parts), k
        assert whole.sumsq[k] == sum(p.sumsq[k] for p in parts), k
    for f in ("steps", "events", "reincidences", "capped", "trapped", "n"):
        assert getattr(whole, f) == sum(getattr(p, f) for p in parts), f
    r = tally_to_result(whole)
    z = cases.zscores(r.mean, r.se, c["mean"], c["se"])
    assert max(abs(x) for x in z) <= 3.0, (z, r.mean, c["mean"])


def test_lookup_workload_full_instance_count(engine):
    from ismc_gb300.workloads import lookup_grid
    insts = lookup_grid(seed=2, scale=1e-2)
    assert len(insts) == 64 * 64 + 512
    batch = engine.run_batch_raw(insts)
    assert all(t.status == 0 and t.n == i.n_packets for t, i in zip(batch, insts))
    rng = np.random.default_rng(8)
    sample = sorted(set(rng.choice(len(insts), 24, replace=False).tolist()) | {0, len(insts) - 1})
    for k in sample:
        alone = engine.run_batch_raw([insts[k]])[0]
        assert _same(batch[k], alone), k


def test_instance_above_the_per_instance_limit(engine):
    """5e9 packets of the multilayer benchmark stack in one Engine.run_batch
    call: above ISMC_MAX_PACKETS (2^31), so the API runs three consecutive
    packet ranges in one launch and adds their tallies as Python integers
    (the A sum alone passes 2^63).  The merged means agree with the
    reference's own runs within 3 combined standard errors, and their
    standard errors are sqrt(50) times smaller than those of a 1e8 run."""
    c = cases.golden()["bench1_multilayer"]
    N = 5_000_000_000
    inst = cases.case_instance(c, N, seed=77)
    r = engine.run_batch([inst])[0]
    assert r.status == 0 and r.n == N
    assert r.sums[0] > 2 ** 63
    z = cases.zscores(r.mean, r.se, c["mean"], c["se"])
    assert max(abs(x) for x in z) <= 3.0, z
    small = engine.run_batch([cases.case_instance(c, 100_000_000, seed=77)])[0]
    for k in (1, 3):
        assert abs(small.se[k] / r.se[k] / np.sqrt(50) - 1) < 0.05
