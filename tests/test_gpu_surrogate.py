"""What the trained surrogate gains the inverse solver.

A small network is trained on the GPU from batched Monte Carlo data (the
benchmark's pipeline at reduced size), then the same synthetic measurements
are solved three ways:

  plain      PRAXIS on 1e5-packet Monte Carlo objectives (ismc_solve_batch)
  trained    surrogate proposal + Gauss-Newton + 1e6-packet MC verification,
             offset correction and PRAXIS fallback (surrogate_solve)
  untrained  the same surrogate path with the network at its initial weights

The trained surrogate must need several times fewer Monte Carlo packets per
solve than the plain path and than the untrained network (whose proposals
fail verification and fall back), while its answers stay as close to the
truth as the plain path's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIG = np.array([0.002, 0.002, 0.0005])


@pytest.fixture(scope="module")
def setup():
    from ismc_gb300 import Engine, build
    from ismc_gb300.benchmarks import SOLVE_LO, SOLVE_HI, make_measurements
    from ismc_gb300.surrogate import Surrogate, sample_inputs, simulate
    build.build()
    eng = Engine(0)
    X = sample_inputs(65536, seed=1)
    Y, _ = simulate(eng, X, 20_000, seed=1)
    trained = Surrogate(0, max_batch=4096, seed=1)
    trained.train(X.astype(np.float32), Y.astype(np.float32), epochs=150, batch=4096, lr=1e-3)
    untrained = Surrogate(0, max_batch=4096, seed=1)
    truth, meas = make_measurements(eng, 48, seed=11)
    yield eng, trained, untrained, truth, meas
    trained.close()
    untrained.close()
    eng.close()


def test_trained_surrogate_gains_over_plain_and_untrained(setup):
    from ismc_gb300.api import make_solve
    from ismc_gb300.benchmarks import SOLVE_LO, SOLVE_HI
    from ismc_gb300.surrogate import sample_stack, surrogate_solve
    from ismc_gb300.workloads import bench_spheres
    eng, trained, untrained, truth, meas = setup
    k = 16
    reqs = [make_solve(sample_stack(1.0, 10.0, 0.9, 0.1, 1.4), 1, bench_spheres(), 100_000,
                       (meas[i, 0], None, meas[i, 1], meas[i, 2]), x0=(0.3, 10.0), seed=100 + i,
                       lo=SOLVE_LO, hi=SOLVE_HI, max_evals=400) for i in range(k)]
    outp = eng.solve_batch(reqs)
    xp = np.array([[o.x[0], o.x[1]] for o in outp])
    plain_packets = np.mean([o.evals for o in outp]) * 100_000

    rt = surrogate_solve(trained, eng, meas, SIG, seed=5)
    ru = surrogate_solve(untrained, eng, meas, SIG, seed=5)
    per_t = rt["mc_packets"] / len(meas)
    per_u = ru["mc_packets"] / len(meas)
    # the gain: Monte Carlo work per solve
    assert per_t * 4 < plain_packets, (per_t, plain_packets)
    assert per_t * 3 < per_u, (per_t, per_u, rt["fallback"].mean(), ru["fallback"].mean())
    assert rt["fallback"].mean() < ru["fallback"].mean()
    # and the answers are as close to the truth as the plain path's.  (The two
    # paths are compared through the truth: with 1e5-packet objectives the
    # plain answers themselves scatter by several percent in mu_a.)
    es = np.abs(rt["x"] / truth - 1)
    ep = np.abs(xp / truth[:k] - 1)
    assert np.median(es[:, 1]) < 0.05, es
    assert np.median(es[:, 0]) < 0.20, es
    assert np.all(np.median(es[:k], 0) <= 1.5 * np.median(ep, 0) + 0.02), (es[:k], ep)
    # verified points reproduce the measurements within 3 sigma where accepted
    ok = ~rt["fallback"]
    miss = np.abs(rt["verified"][ok] - meas[ok]) > 3 * np.sqrt(SIG ** 2 + rt["verified_se"][ok] ** 2)
    assert not miss.any()
