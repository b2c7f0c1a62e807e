"""Edge cases of the propagator, bit-exact against the FP32 twin
(oracle/ismc_twin.c) through the C ABI: the largest stack the ABI holds,
packet ids above 2^32, a single packet, one-layer slabs with and without
spheres, non-scattering layers only, and the batch-size limits."""
import ctypes as C

import pytest

import cases
import oracle
from ismc_gb300 import Layer, Spheres, _abi, make_instance
from ismc_gb300.workloads import bench_spheres

pytestmark = pytest.mark.gpu


def _same(a, b):
    return (list(a.sum) == list(b.sum) and list(a.sumsq) == list(b.sumsq) and a.steps == b.steps
            and a.events == b.events and a.reincidences == b.reincidences and a.capped == b.capped
            and a.trapped == b.trapped and a.n == b.n)


def _check(engine, inst):
    g = engine.run_batch_raw([inst])[0]
    t = oracle.twin_run(inst)
    assert g.status == 0
    assert _same(g, t), (list(g.sum), list(t.sum), g.steps, t.steps)
    return g


@pytest.mark.parametrize("mode", ["compat", "physical"])
def test_sixteen_layer_stack(engine, mode):
    """ISMC_MAXL = 16 layers: two slides around 14 tissue layers."""
    tissue = [Layer(1.33 + 0.01 * k, 0.1 + 0.2 * k, 20.0 + 7.0 * k, 0.6 + 0.02 * k, 0.01 + 0.003 * k)
              for k in range(14)]
    layers = [Layer.slide(1.52, 0.1)] + tissue + [Layer.slide(1.5, 0.12)]
    assert len(layers) == 16
    g = _check(engine, make_instance(layers, bench_spheres(), 20000, seed=5, mode=mode))
    assert g.steps > 0


@pytest.mark.parametrize("mode", ["compat", "physical"])
@pytest.mark.parametrize("name", sorted(cases.extreme_stacks()))
def test_extreme_stacks(engine, name, mode):
    """Anisotropy extremes (g = -0.9, 0.99, 1, 0) with index-matched layers,
    and strong index contrast with a 20 um layer, a strong absorber and
    large ports (tests/cases.py extreme_stacks)."""
    layers, sph = cases.extreme_stacks()[name]
    g = _check(engine, make_instance(layers, sph, 20000, seed=21, mode=mode))
    assert g.steps > 0


def test_packet_ids_above_2_pow_32(engine):
    """Packet ids feed two counter words of Philox: ranges crossing 2^32 and far
    above it are drawn exactly as the twin draws them."""
    layers = [Layer.slide(1.5, 0.1), Layer(1.4, 1.0, 100.0, 0.9, 0.1), Layer.slide(1.5, 0.1)]
    for off in ((1 << 32) - 7000, (1 << 40) + 12345):
        _check(engine, make_instance(layers, bench_spheres(), 15000, seed=8, packet_offset=off))


def test_single_packet_and_single_slab(engine):
    slab = [Layer(1.4, 0.5, 50.0, 0.8, 0.2)]
    _check(engine, make_instance(slab, bench_spheres(), 1, seed=3))
    no_spheres = Spheres(R=False, T=False)
    _check(engine, make_instance(slab, no_spheres, 30000, seed=4))
    r_only = Spheres(R=True, T=False)
    _check(engine, make_instance(slab, r_only, 30000, seed=4, roulette_threshold=1e-3))


def test_non_scattering_stack(engine):
    """Only slides: no photon steps; every packet ends as specular, unscattered
    transmission or absorption in the glass (physical mode)."""
    glass = [Layer(1.5, 0.0, 0.0, 0.0, 0.1), Layer(1.45, 0.0, 0.0, 0.0, 0.2)]
    g = _check(engine, make_instance(glass, bench_spheres(), 20000, seed=6))
    assert g.steps == 0
    _check(engine, make_instance([Layer(1.5, 0.7, 0.0, 0.0, 0.3)], bench_spheres(), 20000, seed=6,
                                 mode="physical"))


def test_batch_size_limits(engine):
    """An empty batch is an argument error; a batch of many one-packet
    instances runs each exactly once."""
    lib = engine.lib
    out = _abi.Tally()
    rc = lib.ismc_run_batch(engine.h, None, 0, None, C.byref(out))
    assert rc == -1
    layers = [Layer(1.4, 1.0, 30.0, 0.7, 0.05)]
    insts = [make_instance(layers, bench_spheres(), 1, seed=11, stream=k) for k in range(5000)]
    res = engine.run_batch_raw(insts)
    assert all(t.n == 1 and t.status == 0 for t in res)
    for k in (0, 1, 2499, 4999):
        assert _same(res[k], oracle.twin_run(insts[k]))


def test_packet_count_beyond_tally_headroom(engine):
    """An instance of more than ISMC_MAX_PACKETS (2^31) packets could wrap its
    64-bit sums.  The host-pointer entry point refuses the batch before any
    launch; the device-pointer entry point runs the rest of the batch and marks
    that instance ISMC_ERR_CAPACITY with n = 0."""
    import torch
    from ismc_gb300 import IsmcError
    good = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], bench_spheres(), 30_000, seed=8)
    big = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1)], bench_spheres(), 5_000_000_000, seed=8)
    with pytest.raises(IsmcError) as e:
        engine.run_batch_raw([good, big])
    assert e.value.code == _abi.ERR_CAPACITY
    arr = (_abi.Instance * 2)(good, big)
    d_in = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).cuda()
    d_out = torch.zeros(2 * C.sizeof(_abi.Tally), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    engine.run_batch_device(d_in.data_ptr(), 2, d_out.data_ptr(), s.cuda_stream)
    s.synchronize()
    out = (_abi.Tally * 2).from_buffer_copy(d_out.cpu().numpy().tobytes())
    assert _same(out[0], oracle.twin_run(good)) and out[0].status == 0
    assert out[1].status == _abi.ERR_CAPACITY and out[1].n == 0 and list(out[1].sum) == [0] * 5
    # the context stays usable
    assert engine.run_batch_raw([good])[0].status == 0


def test_instance_above_the_packet_limit_runs_in_parts(engine):
    """Engine.run_batch runs an instance of more than max_packets packets
    (ISMC_MAX_PACKETS by default) as consecutive packet ranges in the same
    launch.  Every draw is keyed by the packet id, so the merged tallies equal
    one run of the whole range bit for bit."""
    from ismc_gb300.workloads import bench1_layers
    inst = make_instance(bench1_layers(), bench_spheres(), 3_500_000, seed=12, packet_offset=5)
    whole = engine.run_batch([inst])[0]
    parts = engine.run_batch([inst], max_packets=1_000_000)[0]
    assert parts.status == 0
    assert parts.sums == whole.sums and parts.sumsqs == whole.sumsqs
    assert (parts.n, parts.steps, parts.events, parts.reincidences, parts.trapped) == \
        (whole.n, whole.steps, whole.events, whole.reincidences, whole.trapped)
    assert parts.mean == whole.mean and parts.se == whole.se
