"""GPU parity: the CUDA propagator against the oracles, through the C ABI.

1. Bit-exactness: for the same instance the GPU's integer tallies equal the
   FP32 twin's (oracle/ismc_twin.c) exactly -- sums, sums of squares, step,
   event and re-incidence counters -- for every golden case, both modes.
2. Statistics: every tally's GPU mean is within 3 combined standard errors
   of the reference's own Python (tests/golden, 64 seeded batches per case),
   for every golden case, and for the single-layer benchmark configuration at
   its own size (1e5 packets, seed 1234).  The z-scores are listed in the
   terminal summary.
3. Deterministic outputs: specular and ballistic values within 1e-6 relative of
   the FP64 oracle (oracle/analytic64.py).
4. Invariances: launch shape, batching and packet-range sharding never change
   a bit of the result.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import oracle
from conftest import PARITY_Z
from ismc_gb300 import Layer, Spheres, _abi, make_instance, make_tune

pytestmark = pytest.mark.gpu

Z = 3.0
ANALYTIC_RTOL = 1e-6


def _same(a, b):
    return (list(a.sum) == list(b.sum) and list(a.sumsq) == list(b.sumsq) and a.steps == b.steps
            and a.events == b.events and a.reincidences == b.reincidences and a.capped == b.capped
            and a.trapped == b.trapped)


def _diff(a, b):
    return {"sum": (list(a.sum), list(b.sum)), "steps": (a.steps, b.steps),
            "events": (a.events, b.events)}


@pytest.mark.parametrize("mode", ["compat", "physical"])
@pytest.mark.parametrize("name", sorted(cases.golden()))
def test_gpu_bit_exact_vs_twin(engine, name, mode):
    c = cases.golden()[name]
    n = 4000 if name == "grid_high_albedo_thick" else 30000
    inst = cases.case_instance(c, n, seed=424242, mode=mode)
    g = engine.run_batch_raw([inst])[0]
    t = oracle.twin_run(inst)
    assert g.status == 0
    assert _same(g, t), _diff(g, t)


@pytest.mark.parametrize("name", sorted(cases.golden()))
def test_gpu_matches_reference(engine, name):
    c = cases.golden()[name]
    n = 1_000_000 if name == "grid_high_albedo_thick" else 4_000_000
    r = engine.run_batch([cases.case_instance(c, n, seed=31337)])[0]
    z = cases.zscores(r.mean, r.se, c["mean"], c["se"])
    PARITY_Z.append((f"{name} ({n:.0e} packets)", z))
    assert max(abs(x) for x in z) <= Z, f"{name}: z={z} gpu={r.mean} ref={c['mean']}"


def test_gpu_single_layer_configuration_matches_reference(engine):
    """The single-layer benchmark configuration exactly as specified: one slab
    (n 1.4, mua 1, mus 100, g 0.9, d 0.1 cm) between n=1.5 slides, both
    spheres with crosstalk, 1e5 packets, Philox seed 1234, against the
    reference's ISMLMC.py on the same stack."""
    c = cases.golden()["bench0_slides"]
    inst = make_instance(cases.bench0_layers(), cases.bench_spheres(), 100_000, seed=1234,
                         roulette_threshold=1e-4, roulette_m=10.0)
    r = engine.run_batch([inst])[0]
    assert r.status == 0 and r.n == 100_000
    z = cases.zscores(r.mean, r.se, c["mean"], c["se"])
    PARITY_Z.append(("single-layer config (1e5, seed 1234)", z))
    assert max(abs(x) for x in z) <= Z, f"z={z} gpu={r.mean} ref={c['mean']}"


def test_gpu_launch_shape_invariance(engine):
    c = cases.golden()["bench1_multilayer"]
    inst = cases.case_instance(c, 200_000, seed=9)
    ref = engine.run_batch_raw([inst])[0]
    for bt, chunk in ((128, 32), (256, 1000), (512, 96), (384, 65536), (64, 7)):
        got = engine.run_batch_raw([inst], make_tune(bt, 0, chunk, 0))[0]
        assert _same(got, ref), (bt, chunk)
    # a batch below half the tuned launch's lanes runs one packet per lane when
    # no shape is requested: the same tallies as under requested shapes
    small = cases.case_instance(c, 5_000, seed=9)
    auto = engine.run_batch_raw([small])[0]
    for bt in (64, 512):
        assert _same(engine.run_batch_raw([small], make_tune(bt, 0, 0, 0))[0], auto), bt


def test_gpu_uneven_batch_equals_single_runs(engine):
    G = cases.golden()
    rng = np.random.default_rng(4)
    insts = []
    for k, name in enumerate(sorted(G)):
        n = int(rng.integers(0, 60000)) if k != 3 else 0
        insts.append(cases.case_instance(G[name], n, seed=1000 + k, stream=k,
                                         mode="physical" if k % 3 == 0 else "compat"))
    batch = engine.run_batch_raw(insts)
    for inst, b in zip(insts, batch):
        s = engine.run_batch_raw([inst])[0]
        assert _same(b, s)
        assert b.n == inst.n_packets


def test_gpu_sharding_is_exact(engine):
    c = cases.golden()["bench0_slides"]
    whole = engine.run_batch_raw([cases.case_instance(c, 500_000, seed=77)])[0]
    parts = [cases.case_instance(c, 123_457, seed=77),
             cases.case_instance(c, 500_000 - 123_457, seed=77, packet_offset=123_457)]
    a, b = engine.run_batch_raw(parts)
    for k in range(5):
        assert whole.sum[k] == a.sum[k] + b.sum[k]
        assert whole.sumsq[k] == a.sumsq[k] + b.sumsq[k]
    assert whole.steps == a.steps + b.steps


def _analytic_cases():
    yield [Layer.slide(1.5, 0.1), Layer(1.4, 1.0, 100.0, 0.9, 0.1), Layer.slide(1.5, 0.1)]
    yield cases.bench1_layers()
    yield [Layer(1.4, 1.0, 100.0, 0.9, 0.1)]
    yield [Layer(1.33, 0.3, 0.0, 0.0, 0.2), Layer(1.5, 2.0, 0.0, 0.0, 0.5)]
    yield [Layer.slide(1.52, 0.17), Layer(1.37, 0.01, 1.0, 0.9, 0.05), Layer(1.45, 10.0, 5.0, 0.6, 0.2),
           Layer(1.41, 0.4, 40.0, 0.8, 0.31), Layer.slide(1.5, 0.1)]
    yield [Layer(1.5, 0.5, 0.0, 0.0, 0.3)]


@pytest.mark.parametrize("mode", ["compat", "physical"])
def test_gpu_analytic_outputs_vs_fp64(engine, mode):
    for layers in _analytic_cases():
        inst = make_instance(layers, cases.bench_spheres(), 1, seed=1, mode=mode)
        t = engine.run_batch_raw([inst])[0]
        st = inst.stack
        spec, ball = oracle.analytic64(st.n[:st.L], st.mus[:st.L], st.mut[:st.L], st.d[:st.L],
                                       mode=mode)
        assert abs(t.analytic_specular - spec) <= ANALYTIC_RTOL * spec, (layers, spec)
        assert abs(t.analytic_ballistic - ball) <= ANALYTIC_RTOL * ball, (layers, ball)


def test_gpu_ballistic_mc_matches_analytic(engine):
    """Physical mode, no scattering anywhere: every transmitted packet is
    unscattered, so T_u estimates the ballistic transmittance and R_s the
    specular reflectance of the whole stack (3 sigma)."""
    layers = [Layer(1.33, 0.3, 0.0, 0.0, 0.2), Layer(1.5, 2.0, 0.0, 0.0, 0.5),
              Layer(1.45, 0.1, 0.0, 0.0, 0.3)]
    inst = make_instance(layers, cases.bench_spheres(), 2_000_000, seed=5, mode="physical")
    r = engine.run_batch([inst])[0]
    assert abs(r["T_u"] - r.analytic_ballistic) <= 3 * r.se[4]
    assert abs(r["R_s"] - r.analytic_specular) <= 3 * r.se[2]
    assert r["R_d"] == 0.0 and r["T_d"] == 0.0


@pytest.mark.parametrize("name", sorted(cases.extreme_stacks()))
def test_gpu_extreme_stacks_match_fp64_restatement(engine, name):
    """Stacks the golden runs do not reach (tests/cases.py extreme_stacks:
    anisotropy extremes and index-matched layers; strong index contrast,
    a 20 um layer, a strong absorber, large ports): the GPU at 2e6 packets
    against the FP64 restatement of the reference's walk
    (oracle/ismc_ref64.c) at 4e5 packets, within 3 combined standard errors
    per tally.  The GPU's tallies are the twin's bit for bit
    (test_gpu_edges.py), whose CPU test makes the same comparison."""
    layers, sph = cases.extreme_stacks()[name]
    r = engine.run_batch([make_instance(layers, sph, 2_000_000, seed=22)])[0]
    m, se, _ = oracle.ref64_run(make_instance(layers, sph, 400_000, seed=23))
    z = cases.zscores(r.mean, r.se, m, se)
    assert r.status == 0 and max(abs(x) for x in z) <= 3.0, (z, r.mean, m)


@pytest.mark.parametrize("name", sorted(cases.physical_stacks()))
def test_gpu_physical_mode_matches_fp64_physical_walk(engine, name):
    """The physical mode on the GPU (2e6 packets) against the independent
    FP64 physical walk of oracle/ismc_ref64.c (1e6 packets), 3 combined
    standard errors per tally (tests/cases.py physical_stacks: the benchmark
    stack, absorbing slides, strong index contrast, T sphere only)."""
    layers, sph = cases.physical_stacks()[name]
    r = engine.run_batch([make_instance(layers, sph, 2_000_000, seed=22, mode="physical")])[0]
    m, se, _ = oracle.ref64_run(make_instance(layers, sph, 1_000_000, seed=23, mode="physical"))
    z = cases.zscores(r.mean, r.se, m, se)
    assert r.status == 0 and max(abs(x) for x in z) <= 3.0, (z, r.mean, m)


def test_gpu_physical_equals_compat_without_slides_or_spheres(engine):
    """With no slide and no sphere the two modes take identical decisions."""
    sp = Spheres(R=False, T=False)
    inst_c = make_instance(cases.bench1_layers()[1:4], sp, 100_000, seed=3, mode="compat")
    inst_p = make_instance(cases.bench1_layers()[1:4], sp, 100_000, seed=3, mode="physical")
    a, b = engine.run_batch_raw([inst_c, inst_p])
    assert _same(a, b)


def test_gpu_event_cap_reports_status(engine):
    c = cases.golden()["bench1_multilayer"]
    inst = cases.case_instance(c, 5000, seed=2)
    t = engine.run_batch_raw([inst], make_tune(256, 0, 64, 20))[0]
    assert t.status == _abi.ERR_STEP_LIMIT
    assert 0 < t.capped <= 5000
    tw = oracle.twin_run(inst, max_events=20)
    assert _same(t, tw)
    # the context stays usable
    ok = engine.run_batch_raw([inst])[0]
    assert ok.status == 0 and ok.capped == 0


def test_gpu_invalid_instances(engine):
    from ismc_gb300 import IsmcError
    bad = make_instance([Layer(1.4, 1.0, 100.0, 0.9, -0.1)], cases.bench_spheres(), 10, seed=1)
    with pytest.raises(IsmcError) as e:
        engine.run_batch_raw([bad])
    assert e.value.code == _abi.ERR_INVALID_ARG


def test_gpu_device_pointer_entry(engine):
    """ismc_run_batch_device on device-resident instances; an invalid instance
    is flagged per instance by the device-side check."""
    import torch
    c = cases.golden()["slab_both"]
    good = cases.case_instance(c, 50_000, seed=12)
    bad = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], cases.bench_spheres(), 10, seed=1)
    bad.stack.d[0] = float("nan")
    arr = (_abi.Instance * 2)(good, bad)
    raw = bytes(arr)
    d_in = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    d_out = torch.zeros(2 * C.sizeof(_abi.Tally), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    engine.run_batch_device(d_in.data_ptr(), 2, d_out.data_ptr(), s.cuda_stream)
    s.synchronize()
    out = (_abi.Tally * 2).from_buffer_copy(d_out.cpu().numpy().tobytes())
    assert _same(out[0], oracle.twin_run(good))
    assert out[1].status == _abi.ERR_INVALID_ARG and out[1].n == 0
