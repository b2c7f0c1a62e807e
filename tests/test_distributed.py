"""Multi-rank sharding on CPU: two gloo ranks each simulate their packet range
(with the CPU twin standing in for the GPU engine, which has the same integer
tallies), merge with ismc_gb300.distributed.allreduce_tallies, and must equal
a single-process run over the whole range bit for bit."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    import torch.distributed as dist
    import cases
    import oracle
    from ismc_gb300 import distributed as D
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        G = cases.golden()
        insts = [cases.case_instance(G["bench0_slides"], n, seed=5),
                 cases.case_instance(G["five_layer_mixed"], n // 3, seed=6, stream=2)]
        mine = [oracle.twin_run(D.shard_instance(x, rank, world), threads=2) for x in insts]
        merged = D.allreduce_tallies(mine)
        # the check bench.py runs under torchrun, with the twin as the engine
        _, same = D.sharded_run_check(lambda x: oracle.twin_run(x, threads=2),
                                      cases.case_instance(G["bench1_multilayer"], n // 4, seed=7),
                                      rank, world)
        if rank == 0:
            q.put(([(list(m.sum), list(m.sumsq), m.steps, m.events, m.n, m.status) for m in merged],
                   same))
    finally:
        dist.destroy_process_group()


def test_two_rank_merge_equals_single_process():
    import cases
    import oracle
    n = 12_001
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    got, same = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    G = cases.golden()
    whole = [oracle.twin_run(cases.case_instance(G["bench0_slides"], n, seed=5)),
             oracle.twin_run(cases.case_instance(G["five_layer_mixed"], n // 3, seed=6, stream=2))]
    for (s, q2, st, ev, nn, status), w in zip(got, whole):
        assert s == list(w.sum) and q2 == list(w.sumsq)
        assert st == w.steps and ev == w.events and nn == w.n and status == w.status
    assert same is True


def test_shard_range_covers_exactly():
    from ismc_gb300.distributed import shard_range
    for n in (0, 1, 7, 1000, 10**9 + 7):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world, offset=11) for r in range(world)]
            assert ranges[0][0] == 11
            assert sum(c for _, c in ranges) == n
            for (a, c), (b, _) in zip(ranges, ranges[1:]):
                assert a + c == b


def test_bench_reference_arm_under_torchrun_two_ranks():
    """`bench.py --impl reference` launched as the multi-GPU runs launch it
    (torchrun, two ranks, gloo on CPU): rank 0 alone runs the reference and
    prints one JSON line; the other rank exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "1", "--packets", "2000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=root)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
