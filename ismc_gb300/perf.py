"""Evidence behind the propagator's issue-rate roofline.

    python -m ismc_gb300.perf build                  # both tools below, in ismc_gb300/_build/perf/
    python -m ismc_gb300.perf components             # run the building-block kernels once
    python -m ismc_gb300.perf components --csv F     # read an ncu CSV of that run (below)
    python -m ismc_gb300.perf branches [--packets N] [--stacks bench1,bench1_noslides,bench0]

components: csrc/perf/ismc_components.cu runs each building block of an event
(a Philox4x32-10 block, -ln u, sin/cos 2 pi u, an IEEE division and square
root, the interface's reflect-or-transmit draw, the spin) 1024 times per
thread.  Under
    ncu --metrics smsp__inst_executed.sum,smsp__thread_inst_executed.sum \\
        --clock-control none --csv --log-file F ismc_gb300/_build/perf/components
the --csv step turns the counts into warp instructions per call, the loop's
own overhead (k_loop) subtracted.

branches: the library rebuilt with -DISMC_BRANCH_STATS (counters of every
branch of the event loop; never the product build) runs the benchmark stacks
and prints, per branch, warp executions per photon-step and active lanes per
execution.  With the per-call costs this apportions the issue slots of a step.
"""
import argparse
import csv
import ctypes as C
import json
import os
import subprocess
import sys

from . import build as B

OUT = os.path.join(B.BUILD, "perf")
COMPONENTS = os.path.join(OUT, "components")
STATS_LIB = os.path.join(OUT, "libismc_stats.so")
BRANCHES = ("iteration", "handout", "event", "incident", "walk", "interface", "interaction",
            "spin", "sphere", "fin")
# ismc_components.cu's launch: 608 blocks x 256 threads, 1024 calls per thread
_WARPS, _ITERS = 608 * 256 // 32, 1024


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_components():
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(B.CSRC, "perf", "ismc_components.cu")
    flags = [f for f in B.NVCC_FLAGS if not f.startswith("-Xcompiler") and "fPIC" not in f]
    _run([B.nvcc(), src, "-o", COMPONENTS] + flags)
    return COMPONENTS


def build_stats_library():
    """The library with the branch counters compiled into the propagator."""
    os.makedirs(OUT, exist_ok=True)
    objs = []
    for src in B.SOURCES:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        srcp = os.path.join(B.CSRC, src)
        if src.endswith(".cpp"):
            cmd = [os.environ.get("CXX", "g++"), "-c", srcp, "-o", obj] + B.CXX_FLAGS
        else:
            flags = [f for f in B.NVCC_FLAGS if not (src in B.CONTRACTED and f == "-fmad=false")]
            cmd = [B.nvcc(), "-c", srcp, "-o", obj] + flags
            if src == "ismc_kernels.cu":
                cmd.append("-DISMC_BRANCH_STATS")
        objs.append((cmd, obj))
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(len(objs)) as ex:
        list(ex.map(lambda co: _run(co[0]), objs))
    _run([B.nvcc(), "-shared", "-o", STATS_LIB] + [o for _, o in objs] + B.ARCH +
         ["-lcudart", "-lstdc++"])
    return STATS_LIB


def components_from_csv(path):
    """Warp instructions (and active lanes) per call from an ncu CSV of the
    components binary, k_loop's overhead subtracted."""
    rows = list(csv.reader(open(path)))
    hdr, vals = None, {}
    for r in rows:
        if r and r[0] == "ID":
            hdr = r
            continue
        if hdr and len(r) == len(hdr):
            d = dict(zip(hdr, r))
            k = d["Kernel Name"].split("(")[0]
            vals.setdefault(k, {})[d["Metric Name"]] = float(d["Metric Value"].replace(",", ""))
    per = {k: v["smsp__inst_executed.sum"] / (_WARPS * _ITERS) for k, v in vals.items()}
    loop = per.get("k_loop", 0.0)
    out = {}
    for k, v in vals.items():
        if k == "k_loop":
            continue
        lanes = v["smsp__thread_inst_executed.sum"] / v["smsp__inst_executed.sum"]
        out[k[2:]] = {"warp_inst_per_call": per[k] - loop, "lanes": lanes}
    out["_loop_overhead"] = loop
    return out


def branch_stats(stacks=("bench1", "bench1_noslides", "bench0"), packets=4_000_000):
    """Per-branch warp executions per photon-step and active lanes per
    execution, on the benchmark stacks (autotuned launch shape)."""
    from . import api
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    lib = api.load_library(STATS_LIB)
    lib.ismc_branch_stats_read.argtypes = [C.POINTER(C.c_ulonglong)]
    lib.ismc_branch_stats_read.restype = C.c_int
    lib.ismc_branch_stats_reset.restype = C.c_int
    import bench
    eng = api.Engine(0)
    res = []
    for st in stacks:
        inst = bench.workload_instance(packets, stack=st)
        eng.autotune([inst])
        eng.run_batch_raw([inst])
        lib.ismc_branch_stats_reset()
        t = eng.run_batch_raw([inst])[0]
        buf = (C.c_ulonglong * 32)()
        lib.ismc_branch_stats_read(buf)
        row = {"stack": st, "packets": int(t.n), "steps": int(t.steps), "events": int(t.events)}
        for k, name in enumerate(BRANCHES):
            ex, ln = buf[2 * k], buf[2 * k + 1]
            row[name] = {"execs_per_step": ex / max(t.steps, 1), "lanes": ln / max(ex, 1)}
        res.append(row)
    eng.close()
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("what", choices=["build", "components", "branches"])
    ap.add_argument("--csv", default=None)
    ap.add_argument("--packets", type=int, default=4_000_000)
    ap.add_argument("--stacks", default="bench1,bench1_noslides,bench0")
    a = ap.parse_args(argv)
    if a.what == "build":
        print(build_components())
        print(build_stats_library())
    elif a.what == "components":
        if a.csv:
            print(json.dumps(components_from_csv(a.csv), indent=1))
        else:
            print(_run([build_components()]).strip())
    else:
        if not os.path.exists(STATS_LIB):
            build_stats_library()
        for row in branch_stats(tuple(a.stacks.split(",")), a.packets):
            print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
