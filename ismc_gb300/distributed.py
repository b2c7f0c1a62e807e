"""Sharding of one simulation across ranks (one process per GPU).

Packets are independent and every draw is keyed by the packet id, so a rank
simulates the contiguous packet range it owns and the tallies -- 64-bit
integer sums -- are added across ranks.  The merged result is bit-identical
to a single-process run over the whole range, for any number of ranks.  The
only exchange is that sum (one all-reduce of n_inst x 16 int64 words), which
replaces the host-side merge of the reference's multi-GPU lookup generator
(CUDA/ISMLMC-lookup.cu:273-283, one std::async thread per device).
"""
import ctypes as C

from . import _abi

# integer words of ismc_tally that are sums across shards (n .. trapped)
SUM_WORDS = 1 + 5 + 5 + 5


def shard_range(n_packets, rank, world, offset=0):
    """[first, first + count) of rank's share of n_packets packets."""
    lo = offset + n_packets * rank // world
    hi = offset + n_packets * (rank + 1) // world
    return lo, hi - lo


def shard_instance(inst, rank, world):
    """Copy of an instance restricted to rank's packet range."""
    x = _abi.Instance.from_buffer_copy(bytes(inst))
    x.packet_offset, x.n_packets = shard_range(inst.n_packets, rank, world, inst.packet_offset)
    return x


def allreduce_tallies(tallies, group=None):
    """Sum the integer fields of a list of ismc_tally across the process group
    (torch.distributed, gloo on CPU or NCCL on GPU).  Statuses combine by
    minimum (any error wins); analytic values are identical on every rank."""
    import torch
    import torch.distributed as dist
    n = len(tallies)
    words = torch.empty((n, SUM_WORDS), dtype=torch.int64)
    status = torch.empty(n, dtype=torch.int64)
    for i, t in enumerate(tallies):
        raw = (C.c_uint64 * SUM_WORDS).from_buffer_copy(bytes(t)[:8 * SUM_WORDS])
        words[i] = torch.tensor([int(v) if v < 2**63 else int(v) - 2**64 for v in raw],
                                dtype=torch.int64)
        status[i] = int(t.status)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else None
    if dev is not None:
        words, status = words.to(dev), status.to(dev)
    dist.all_reduce(words, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(status, op=dist.ReduceOp.MIN, group=group)
    words, status = words.cpu(), status.cpu()
    out = []
    for i, t in enumerate(tallies):
        m = _abi.Tally.from_buffer_copy(bytes(t))
        raw = (C.c_uint64 * SUM_WORDS)(*[int(v) % 2**64 for v in words[i].tolist()])
        C.memmove(C.addressof(m), raw, 8 * SUM_WORDS)
        m.status = int(status[i])
        out.append(m)
    return out


def tallies_equal(a, b):
    """Bit equality of two tallies' integer fields and status."""
    return bytes(a)[:8 * SUM_WORDS] == bytes(b)[:8 * SUM_WORDS] and int(a.status) == int(b.status)


def sharded_run_check(run, inst, rank, world, group=None):
    """Simulate `inst` sharded over the process group -- each rank runs its
    packet range with `run` (a callable taking one instance and returning its
    ismc_tally) -- and merge the shards with allreduce_tallies.  Rank 0 then
    runs the whole range alone and compares.  Returns (merged tally, True or
    False on rank 0 / None elsewhere)."""
    mine = run(shard_instance(inst, rank, world))
    merged = allreduce_tallies([mine], group)[0]
    same = tallies_equal(merged, run(inst)) if rank == 0 else None
    return merged, same
