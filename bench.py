"""Benchmark of the GB300 photon propagator.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                    [--stack bench1|bench1_noslides|bench0|bench0_noslides]

Workload (one "step"): the three-layer stack between n = 1.52 slides
(n=1.37/1.40/1.44, mua=0.5/2.0/0.2 1/cm, mus=200/120/50 1/cm, g=0.8/0.9/0.75,
d=0.01/0.15/0.3 cm; slides 0.1 cm), two 5.08 cm spheres with 1.27/1.27/0.635 cm
ports and wall reflectance 0.98, crosstalk on, 1e8 photon packets, seed 7 --
one full forward simulation.  Metric: photons/s.  --stack picks another stack
of the same geometry for comparisons (the single-slab configuration, or either
stack without its slides).

GPU arm (default): `value` is timed with CUDA events around the device-pointer
entry point (instances already in HBM); `e2e` times the host-pointer C ABI call
(ismc_run_batch: H2D of the instance, prepare, scan, propagate, D2H of the
tally) with a host clock.  L2 is flushed (a 512 MB write) before every timed
step.  Under torchrun each rank simulates its own packet range of the same
stack (weak scaling), the max time over ranks is reported, and the ranks'
integer tallies are summed into the merged result; a reduced-size sharded run
is checked bit for bit against a single-process run of the same range.

Reference arm (--impl reference): the reference's own ISMLMC.py / MLMC.py on
every host core where oracle/build_ref.py staged them (as --workload refpython,
below), else the reference's algorithm as restated in FP64 C
(oracle/ismc_ref64.c); each step a bounded packet sample of the same workload.
The GPU arm's cpu_baseline is the same reference Python (with the restatement
beside it), or the restatement alone.
Reference CUDA arm (--impl reference --workload refcuda): the reference's own
CUDA kernel and host entry point (CUDA/CUDAISMLMC.h, compiled unmodified from a
staged copy by oracle/build_ref.py) on the same GPU, in calls of 1e7 packets.
Reference Python arm (--impl reference --workload refpython): the reference's
own ISMLMC.py / MLMC.py (staged unmodified by oracle/build_ref.py) on every host
core, one spawned process per core, each step a bounded packet sample (or
--packets per step when given).
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PACKETS = 100_000_000
SEED = 7
L2_FLUSH_BYTES = 512 << 20
ROOFLINE_FILE = os.path.join(ROOT, "profiles", "propagator_bench1_roofline.json")
# packets per call of the reference's CUDA entry point: its curand-state array
# holds RNGS = 2e7 states and N/256 + 1 blocks of 256 threads use one each
# (CUDA/CUDAISMLMC.h:12, 660-683)
REFCUDA_PACKETS_PER_CALL = 10_000_000


def _layers(stack):
    from ismc_gb300 import workloads as W
    if stack == "bench1":
        return W.bench1_layers()
    if stack == "bench1_noslides":
        return W.bench1_layers()[1:4]
    if stack == "bench0":
        return W.bench0_layers()
    if stack == "bench0_noslides":
        return W.bench0_layers()[1:2]
    raise ValueError(f"unknown stack {stack!r}")


STACK_TEXT = {
    "bench1": "3-layer stack between n=1.52 slides (the multilayer benchmark configuration)",
    "bench1_noslides": "the multilayer benchmark's 3 tissue layers without the slides",
    "bench0": "one slab (n 1.4, mua 1, mus 100, g 0.9, d 0.1 cm) between n=1.5 slides "
              "(the single-layer configuration)",
    "bench0_noslides": "the single-layer configuration's slab without the slides",
}


def workload_layers(stack="bench1"):
    return _layers(stack)


def workload_spheres():
    from ismc_gb300 import Spheres
    return Spheres.from_radii(5.08, 1.27, 1.27, 0.635, 0.98, R=True, T=True)


def workload_instance(n, offset=0, stack="bench1"):
    from ismc_gb300 import make_instance
    return make_instance(workload_layers(stack), workload_spheres(), n, seed=SEED, mode="compat",
                         roulette_threshold=1e-4, roulette_m=10.0, packet_offset=offset)


def workload_config(stack="bench1", packets=PACKETS):
    return {"workload": f"{STACK_TEXT[stack]}, two 5.08 cm spheres with crosstalk, "
                        f"{packets:.0e} packets per step", "stack": stack,
            "layers": len(workload_layers(stack)), "packets_per_step": packets, "seed": SEED,
            "mode": "compat", "l2": "flushed (512 MB write) before every timed step"}


CONFIG = workload_config()


def host_cores():
    """Host cores this process may run on (its CPU affinity), for the CPU arms."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index),
                                          f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up can hold up this process's CUDA calls for
            # most of a second: time nothing before its first sample is in
            t0 = time.perf_counter()
            while not self.rows and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace('.', '', 1).isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace('.', '', 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def cpu_baseline(seconds=12.0, stack="bench1"):
    """The reference's algorithm (FP64 restatement of ISMLMC.py) on all host
    cores, on a bounded packet sample of the workload."""
    import oracle
    threads = host_cores()
    n = 20000
    t0 = time.perf_counter()
    oracle.ref64_run(workload_instance(n, stack=stack), threads=threads)
    dt = time.perf_counter() - t0
    n2 = max(n, int(n * seconds / max(dt, 1e-3)))
    t0 = time.perf_counter()
    _, _, steps = oracle.ref64_run(workload_instance(n2, stack=stack), threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n2 / dt, "unit": "photons/s", "cores": threads, "kind": "port",
            "sample": f"{n2} packets of the workload (FP64 C restatement of ISMLMC.py/MLMC.py, "
                      f"{threads} threads, {dt:.1f} s)", "steps_per_s": steps / dt}


def cpu_solve_baseline(engine, seconds=150.0, packets=100_000, solves=10):
    """The reference's Python minimisation path (minimization.py:199-271:
    scipy Powell on the reference's cost, one N-packet forward run per
    objective) with the FP64 restatement of ISMLMC.py on all host cores as
    the forward model, on the first `solves` of the solve benchmark's
    measurements, stopping early after about `seconds`.  Reported beside the
    GPU paths."""
    import math
    import numpy as np
    from scipy.optimize import minimize
    import oracle
    from ismc_gb300 import make_instance
    from ismc_gb300.benchmarks import make_measurements
    from ismc_gb300.surrogate import sample_stack
    from ismc_gb300.workloads import bench_spheres
    threads = host_cores()
    sph = bench_spheres()
    truth, meas = make_measurements(engine, solves, seed=4)
    evals = [0]

    def cost(x, m, k):
        mua, musr = float(x[0]), float(x[1])
        if not (mua > 0.0 and musr > 0.0):
            return 1e3                        # outside the physical range
        evals[0] += 1
        inst = make_instance(sample_stack(mua, musr, 0.9, 0.1, 1.4), sph, packets, seed=900 + k,
                             stream=evals[0], mode="compat")
        mean, _, _ = oracle.ref64_run(inst, threads=threads)
        rd, td, tu = mean[1], mean[3], mean[4]
        return math.sqrt(((rd - m[0]) / m[0]) ** 2 + ((td - m[1]) / m[1]) ** 2 + (tu - m[2]) ** 2)

    t0 = time.perf_counter()
    done, errs = 0, []
    for k in range(len(meas)):
        if done and time.perf_counter() - t0 > seconds:
            break
        res = minimize(cost, [0.3, 10.0], args=(meas[k], k), method="Powell", tol=1e-3,
                       options={"maxfev": 400})
        errs.append([abs(res.x[0] / truth[k, 0] - 1), abs(res.x[1] / truth[k, 1] - 1)])
        done += 1
    dt = time.perf_counter() - t0
    out = {"value": done / dt, "unit": "solves/s", "cores": threads, "kind": "port",
           "sample": f"{done} solves of the benchmark's measurements, scipy Powell (tol 1e-3, at most "
                     f"400 evaluations) on the reference's cost with {packets}-packet FP64 C "
                     f"restatement runs ({threads} threads), {evals[0]} evaluations, {dt:.1f} s",
           "rel_err_vs_truth_median": np.median(np.array(errs), 0).tolist()}
    # The same objective on the reference's own Python forward model: one
    # N-packet ISMLMC() run at each solved measurement's truth, spread over
    # every core, scaled by the evaluations per solve that Powell took above
    from oracle import build_ref, refpython
    model = build_ref.staged_python()
    if model and done:
        S = refpython.sphere_dict(sph)
        per = math.ceil(packets / threads)
        walls = []
        with refpython.Runner(model, threads) as pool:
            pool.run(refpython.layer_tuples(sample_stack(1.0, 10.0, 0.9, 0.1, 1.4)), S, 10, 1)
            for k in range(done):
                L = refpython.layer_tuples(sample_stack(truth[k, 0], truth[k, 1], 0.9, 0.1, 1.4))
                walls.append(pool.run(L, S, per, 100 + k)[1])
        t_obj = sum(walls) / len(walls)
        eps = evals[0] / done
        out["reference_python"] = {
            "objective_s": t_obj, "evals_per_solve": eps,
            "solves_per_s_extrapolated": 1.0 / (eps * t_obj),
            "sample": f"{per * threads}-packet runs of the reference's ISMLMC.py at {done} truths "
                      f"({threads} processes), mean {t_obj:.2f} s per objective, times the "
                      f"{eps:.0f} Powell evaluations per solve measured on the restatement"}
    return out


def cpu_tables_baseline(data, N=1000, M=100, cells_sample=300, seed=3):
    """The reference's makelookup on the host (lookup.py:301-376): scipy's cubic
    griddata for the four tables (timed in full), and the Python Monte Carlo
    uncertainty loop restated in oracle/table64.py, timed on a sample of the
    covered cells and scaled to all of them (the full loop runs for hours)."""
    import numpy as np
    from scipy.interpolate import griddata
    import oracle.table64 as t64
    Rd, Rs, Td, Ts, mu_a, mus_r = data
    I, J = np.meshgrid(np.arange(1, Rd.shape[0]), np.arange(1, Rd.shape[1]), indexing="ij")
    R, T = 100 * Rd[I, J].ravel(), 100 * Td[I, J].ravel()
    o = np.lexsort((T, R))
    P = np.stack([R[o], T[o]], 1)
    g = np.linspace(0, 100, N)
    GX, GY = np.meshgrid(g, g, indexing="ij")
    t0 = time.perf_counter()
    tabs = [griddata(P, v[o], (GX, GY), method="cubic") for v in
            (mu_a[I].ravel(), mus_r[J].ravel(), 100 * Rs[I, J].ravel(), 100 * Ts[I, J].ravel())]
    t_grid = time.perf_counter() - t0
    ok = np.argwhere(np.isfinite(tabs[2]) & np.isfinite(tabs[3]) & (tabs[2] >= 0) & (tabs[3] >= 0))
    rng = np.random.default_rng(seed)
    pick = ok[rng.choice(len(ok), size=min(cells_sample, len(ok)), replace=False)]
    t1 = time.perf_counter()
    t64.uncertainty_map(tabs[0], tabs[1], tabs[2], tabs[3], M, seed,
                        cells=[(int(i), int(j)) for i, j in pick])
    per_cell = (time.perf_counter() - t1) / max(len(pick), 1)
    total = t_grid + per_cell * len(ok)
    return {"value": total, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"scipy griddata(cubic) x4 at {N}x{N}: {t_grid:.1f} s measured; uncertainty "
                      f"loop (M={M}) measured on {len(pick)} of {len(ok)} cells, "
                      f"{per_cell * 1e3:.2f} ms per cell, scaled",
            "griddata_s": t_grid, "uncertainty_s_scaled": per_cell * len(ok)}


def cpu_lookup_baseline(r, seconds=20.0, sample=64, ref_seconds=30.0):
    """The FP64 restatement of the reference on a stratified sample of the
    lookup workload's instances (every k-th of the 4608, budgets capped so the
    sample takes about `seconds`), on all host cores; the full workload's CPU
    time is extrapolated from its photon-step count."""
    import copy
    import oracle
    from ismc_gb300.workloads import lookup_grid
    insts = lookup_grid(seed=2, scale=r.get("scale", 1.0))
    stride = max(1, len(insts) // sample)
    pick = [copy.copy(insts[i]) for i in range(0, len(insts), stride)][:sample]
    threads = host_cores()
    cap = 2000
    t0 = time.perf_counter()
    for x in pick[:8]:
        x2 = copy.copy(x)
        x2.n_packets = min(int(x.n_packets), cap)
        oracle.ref64_run(x2, threads=threads)
    per = (time.perf_counter() - t0) / 8
    cap = max(1000, int(cap * seconds / max(per * len(pick), 1e-3)))
    packets = steps = 0
    t0 = time.perf_counter()
    for x in pick:
        x.n_packets = min(int(x.n_packets), cap)
        _, _, st = oracle.ref64_run(x, threads=threads)
        packets += int(x.n_packets)
        steps += st
    dt = time.perf_counter() - t0
    sps = steps / dt
    out = {"value": packets / dt, "unit": "photons/s", "cores": threads, "kind": "port",
           "steps_per_s": sps,
           "sample": f"{len(pick)} instances (every {stride}th of the workload), at most {cap} packets "
                     f"each, FP64 C restatement on {threads} threads, {dt:.1f} s",
           "full_workload_s_extrapolated": r["steps_per_s"] * r["seconds"] / sps}
    # The reference's own Python on the same instances; the restatement runs
    # the very same instances and packet counts again, and the ratio of the
    # two times scales the extrapolated full-workload time
    from oracle import build_ref, refpython
    model = build_ref.staged_python()
    if model:
        args = [refpython.instance_args(x) for x in pick]
        with refpython.Runner(model, threads) as pool:
            pool.run(*args[0], 1, 1)
            probe = 200
            t0 = time.perf_counter()
            for a in args[:8]:
                pool.run(*a, probe, 3)
            per = (time.perf_counter() - t0) / 8 / probe     # s per packet of one process
            each = max(probe, int(ref_seconds / max(per * len(args), 1e-9)))
            t0 = time.perf_counter()
            for k, a in enumerate(args):
                pool.run(*a, each, 100 + k)
            dt_r = time.perf_counter() - t0
        t0 = time.perf_counter()
        for x in pick:
            x.n_packets = each * threads
            oracle.ref64_run(x, threads=threads)
        dt_p = time.perf_counter() - t0
        out["reference_python"] = {
            "value": each * threads * len(args) / dt_r, "unit": "photons/s",
            "sample": f"the same {len(args)} instances at {each * threads} packets each, the "
                      f"reference's ISMLMC.py in {threads} processes, {dt_r:.1f} s; the "
                      f"restatement on the same packets {dt_p:.2f} s",
            "time_vs_restatement": dt_r / dt_p,
            "full_workload_s_extrapolated": out["full_workload_s_extrapolated"] * dt_r / dt_p}
    return out


def run_dropin_workload(calls=200, N=10_000):
    """The reference's Python drivers call ISMC() once per grid point or
    objective (lookup.py:238, minimization.py:205).  Times that call through
    the drop-in module (GPU) for the config-0 slab, and the same call on the
    FP64 restatement of ISMC.py on one core (the reference's Python is serial)."""
    import oracle
    import ismc_gb300.dropin.ISMC as D
    from ismc_gb300 import make_instance
    from ismc_gb300.workloads import bench_spheres
    sp = bench_spheres()
    args = (1.4, 0.9, 0.1, 1.0, 100.0, 101.0, True, sp.R_pw, sp.R_fs, sp.R_fp, sp.R_fd, sp.R_f,
            sp.R_angle, False, True, sp.T_pw, sp.T_fs, sp.T_fp, sp.T_fd, sp.T_f, sp.T_angle)
    for _ in range(5):
        D.ISMC(N, *args)
    t0 = time.perf_counter()
    for _ in range(calls):
        D.ISMC(N, *args)
    dt = (time.perf_counter() - t0) / calls
    from ismc_gb300 import Layer
    inst = make_instance([Layer(1.4, 1.0, 100.0, 0.9, 0.1, 101.0)], sp, N, seed=1,
                         roulette_threshold=1e-3)
    t0 = time.perf_counter()
    oracle.ref64_run(inst, threads=1)
    dt_cpu = time.perf_counter() - t0
    line = {"metric": "ISMC() calls/s", "value": 1.0 / dt, "unit": "calls/s", "workload": "dropin",
            "config": {"workload": "drop-in ISMC() on the bare config-0 slab (n 1.4, mu_a 1, "
                                   "mu_s 100, g 0.9, d 0.1 cm), both spheres", "packets_per_call": N,
                       "calls": calls},
            "result": {"seconds_per_call": dt},
            "cpu_baseline": {"value": 1.0 / dt_cpu, "unit": "calls/s", "cores": 1, "kind": "port",
                             "sample": f"one {N}-packet call of the FP64 restatement of ISMC.py, "
                                       f"{dt_cpu:.2f} s"}}
    print(json.dumps(line), flush=True)


def load_measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def load_roofline_profile():
    try:
        with open(ROOFLINE_FILE) as fh:
            return json.load(fh)
    except Exception:
        return None


# ----------------------------------------------------------------------------
def run_reference(args, rank, world):
    """The reference arm: the reference's own ISMLMC.py where
    oracle/build_ref.py staged it (steps sized so the whole run takes about
    2.5 minutes), else the FP64 C restatement (oracle/ismc_ref64.c)."""
    if rank != 0:
        return
    from oracle import build_ref
    if build_ref.staged_python():
        run_refpython(args, rank,
                      step_seconds=min(8.0, max(2.0, 150.0 / (args.steps + max(args.warmup, 1)))))
        return
    import oracle
    oracle.lib()
    threads = host_cores()
    # size one step to ~10 s of host work
    n = 20000
    st = args.stack
    t0 = time.perf_counter()
    oracle.ref64_run(workload_instance(n, stack=st), threads=threads)
    dt = time.perf_counter() - t0
    per_step = max(n, int(n * 10.0 / max(dt, 1e-3)))
    for w in range(args.warmup):
        oracle.ref64_run(workload_instance(min(per_step, 20000), offset=w * per_step, stack=st),
                         threads=threads)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        oracle.ref64_run(workload_instance(per_step, offset=k * per_step, stack=st),
                         threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = per_step * args.steps / total
    line = {"metric": "photons/s", "value": value, "unit": "photons/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": dict(workload_config(st, args.packets), packets_per_step=per_step,
                           note="each step is a bounded packet sample of the workload"),
            "cpu_baseline": {"value": value, "unit": "photons/s", "cores": threads, "kind": "port",
                             "sample": f"{per_step} packets per step, FP64 C restatement of "
                                       f"ISMLMC.py/MLMC.py on {threads} threads"},
            "e2e": {"value": value, "unit": "photons/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def refpython_baseline(seconds=12.0, stack="bench1"):
    """The reference's own ISMLMC.py (staged by oracle/build_ref.py) on every
    host core, on a bounded packet sample of the workload (about `seconds` of
    every core's time); None where it was not staged."""
    from oracle import build_ref, refpython
    model = build_ref.staged_python()
    if not model:
        return None
    procs = host_cores()
    layers = refpython.layer_tuples(workload_layers(stack))
    sph = refpython.sphere_dict(workload_spheres())
    with refpython.Runner(model, procs) as pool:
        pool.run(layers, sph, 10, SEED)
        probe = 500
        _, _, c = pool.run(layers, sph, probe, SEED + 1000)
        per_worker = max(probe, int(probe * seconds * procs / max(c, 1e-3)))
        _, wall, _ = pool.run(layers, sph, per_worker, SEED + 100000)
    n = per_worker * procs
    return {"value": n / wall, "unit": "photons/s", "cores": procs, "kind": "reference",
            "sample": f"{n} packets of the workload ({per_worker} on each of {procs} processes), "
                      f"the reference's ISMLMC.py, {wall:.1f} s"}


def run_refpython(args, rank, step_seconds=8.0):
    """The reference's own Python forward model on every host core (--impl
    reference --workload refpython, and the reference arm itself where the
    model was staged): ISMLMC() of the unmodified ISMLMC.py / MLMC.py that
    oracle/build_ref.py stages, one spawned process per core, each step a
    bounded packet sample of the chosen stack (about step_seconds of every
    core's time) unless --packets is given (oracle/refpython.py)."""
    if rank != 0:
        return
    st = args.stack
    base = {"impl": "reference", "metric": "photons/s", "unit": "photons/s",
            "config": workload_config(st, args.packets)}
    if args.workload == "refpython":
        base["workload"] = "refpython"
    from oracle import build_ref, refpython
    model = build_ref.staged_python()
    if not model:
        print(json.dumps(dict(base, unavailable="the reference's Python model was not staged into "
                              "oracle/_ref/python (oracle/build_ref.py stage())")), flush=True)
        return
    procs = host_cores()
    layers = refpython.layer_tuples(workload_layers(st))
    sph = refpython.sphere_dict(workload_spheres())
    explicit = args.packets != PACKETS
    with refpython.Runner(model, procs) as pool:
        # start the workers; without an explicit --packets, size one step to
        # about 8 s of every core's time from the CPU seconds of a probe
        pool.run(layers, sph, 10, SEED)
        probe = 500
        for w in range(max(args.warmup, 1)):
            _, _, c = pool.run(layers, sph, probe, SEED + 1000 * (w + 1))
        if explicit:
            per_worker = max(1, math.ceil(args.packets / procs))
        else:
            per_worker = max(probe, int(probe * step_seconds * procs / max(c, 1e-3)))
        times, cpu, batches = [], 0.0, []
        for k in range(args.steps):
            _, wall, c = pool.run(layers, sph, per_worker, SEED + 100000 * (k + 1))
            times.append(wall)
            cpu += c
            batches += pool.last_batches
    total = sum(times)
    per_step = per_worker * procs
    value = per_step * args.steps / total
    # every worker's share is an independent batch of the reference's run
    K = len(batches)
    mean = [sum(b[i] for b in batches) / K for i in range(5)]
    se = [math.sqrt(sum((b[i] - mean[i]) ** 2 for b in batches) / (K - 1) / K) if K > 1 else None
          for i in range(5)]
    line = dict(base, value=value, n_gpus=int(os.environ.get("WORLD_SIZE", "1")),
                steps=args.steps, warmup=args.warmup,
                ms_per_step=1000 * total / args.steps, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f64", data="synthetic",
                config=dict(base["config"], packets_per_step=per_step,
                            note=("--packets per step, split over the processes" if explicit else
                                  "each step is a bounded packet sample of the workload")),
                cpu_baseline={"value": value, "unit": "photons/s", "cores": procs,
                              "kind": "reference",
                              "sample": f"{per_step} packets per step ({per_worker} on each of "
                                        f"{procs} processes), the reference's ISMLMC.py"},
                e2e={"value": value, "unit": "photons/s", "h2d_bytes_per_step": 0,
                     "d2h_bytes_per_step": 0},
                result={"tallies": ["A", "R_d", "R_s", "T_d", "T_u"], "mean": mean,
                        "se": se, "batches": K,
                        "photons_per_cpu_second": per_step * args.steps / max(cpu, 1e-9)})
    print(json.dumps(line), flush=True)


def run_refcuda(args, rank):
    """The reference's own CUDA forward model on this GPU (--impl reference
    --workload refcuda): kernel CUDAISMLMC timed alone with CUDA events, and the
    reference's host entry point ISMLMC() timed with a host clock, both on the
    chosen stack, in calls of 1e7 packets (oracle/refcuda_bench.cu)."""
    if rank != 0:
        return
    st = args.stack
    base = {"impl": "reference", "workload": "refcuda", "metric": "photons/s", "unit": "photons/s",
            "config": workload_config(st, args.packets)}
    if st not in ("bench1_noslides", "bench0_noslides"):
        # an FP32 rounding artefact of the reference's Fresnel/Snell chain
        # (CUDA/CUDAISMLMC.h:79-96, 71-76) leaves a packet that enters a slide
        # from tissue at |mu_z| < ~2.4e-4 totally reflected at both slide
        # faces; its loop (CUDAISMLMC.h:178-262) ends only when curand_uniform
        # returns exactly 1.0f, about once in 2^25 draws, so a call on a stack
        # with slides runs for an unbounded time
        print(json.dumps(dict(base, unavailable=(
            "the reference's CUDA kernel is timed only on stacks without slides: a packet "
            "entering a slide near grazing is trapped by FP32 total reflection at both faces and "
            "loops until curand returns exactly 1.0f (~2^25 draws)"))), flush=True)
        return
    try:
        from oracle import build_ref
        exe = build_ref.build_refcuda()
    except RuntimeError as e:
        print(json.dumps(dict(base, unavailable="reference CUDA build failed: " +
                              str(e).splitlines()[0])), flush=True)
        return
    if not exe:
        print(json.dumps(dict(base, unavailable="the reference's CUDA sources were not staged into "
                              "oracle/_ref/src (oracle/build_ref.py stage())")), flush=True)
        return
    layers = workload_layers(st)
    sp = workload_spheres()
    per_call = min(REFCUDA_PACKETS_PER_CALL, args.packets)
    calls_per_step = max(1, math.ceil(args.packets / per_call))
    calls = calls_per_step * args.steps

    def arr(xs):
        return " ".join(f"{x:.9g}" for x in xs)

    cmd = [exe, "--layers", str(len(layers)), "-n", arr(l.n for l in layers),
           "-g", arr(l.g for l in layers), "-t", arr(l.d for l in layers),
           "--mua", arr(l.mua for l in layers), "--mus", arr(l.mus for l in layers),
           "--Rsphere", arr((sp.R_pw, sp.R_fs, sp.R_fp, sp.R_fd)),
           "--Tsphere", arr((sp.T_pw, sp.T_fs, sp.T_fp, sp.T_fd)),
           "--packets", str(per_call), "--calls", str(calls)]
    with ClockSampler(0) as clk:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"refcuda_bench failed ({r.returncode}): {r.stderr[-2000:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    packets = per_call * calls
    kern = sum(out["kernel_s"])
    e2e = sum(out["e2e_s"])
    value = packets / kern
    line = dict(base, value=value, n_gpus=1, steps=args.steps, warmup=1,
                ms_per_step=1000 * kern / args.steps, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f32", data="synthetic",
                e2e={"value": packets / e2e, "unit": "photons/s",
                     "api": "the reference's ISMLMC() (CUDA/CUDAISMLMC.h:656-755), host clock"},
                clocks=clk.summary(),
                result={"packets_per_call": per_call, "calls_per_step": calls_per_step,
                        "kernel_mean": out["kernel_mean"], "e2e_mean": out["e2e_mean"],
                        "registers": out["registers"], "launch": f"{out['blocks']} x {out['threads']}",
                        "kernel_s": out["kernel_s"], "e2e_s": out["e2e_s"]},
                note="value: the reference's kernel alone (CUDA events, device-resident arrays, "
                     "its own launch shape); warm-up: one untimed ISMLMC() call that initialises "
                     "the curand states.  Its roulette never lets a packet survive "
                     "(CUDAISMLMC.h:275: integer 1/m = 0) and its tallies are float atomics.")
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, dist):
    import torch
    from ismc_gb300 import Engine, _abi, build
    build.build()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    eng = Engine(dev)
    n = args.packets
    st = args.stack
    inst = workload_instance(n, offset=rank * n, stack=st)
    # the autotuner picks block size and queue chunking on short trial launches
    # of the same workload (kept in the context for every launch below)
    tuned = eng.autotune([inst])
    raw = bytes(inst)
    d_in = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(f"cuda:{dev}")
    d_out = torch.zeros(C.sizeof(_abi.Tally), dtype=torch.uint8, device=f"cuda:{dev}")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    def device_step():
        eng.run_batch_device(d_in.data_ptr(), 1, d_out.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()

    # ---- device-resident timing (CUDA events on the launching stream)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            ev[k][0].record(stream)
            device_step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    dev_time = sum(ms) / 1000.0
    tally = (_abi.Tally).from_buffer_copy(d_out.cpu().numpy().tobytes())
    if tally.status != 0:
        raise RuntimeError(f"propagator status {tally.status}")

    # ---- end-to-end through the host-pointer C ABI (ismc_run_batch)
    e2e_times = []
    res = None
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        res = eng.run_batch([inst])[0]
        e2e_times.append(time.perf_counter() - t0)
    barrier()
    e2e_time = sum(e2e_times)

    merge = None
    if dist is not None:
        t = torch.tensor([dev_time, e2e_time], dtype=torch.float64, device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_time, e2e_time = float(t[0]), float(t[1])
        # the one data exchange of a sharded run: the ranks' integer tallies are
        # summed into the result of the whole packet range [0, world n) ...
        from ismc_gb300 import distributed as D
        from ismc_gb300 import tally_to_result
        merged = D.allreduce_tallies([tally])[0]
        res = tally_to_result(merged)
        # ... and, at a reduced size, that sum equals one process's run of the
        # same range bit for bit
        check_n = min(n * world, 2_000_000)
        _, same = D.sharded_run_check(lambda x: eng.run_batch_raw([x])[0],
                                      workload_instance(check_n, stack=st), rank, world)
        merge = {"merged_packets": int(merged.n), "check_packets": check_n,
                 "sharded_equals_single_process": same}
    if rank != 0:
        return
    total_packets = n * args.steps * world
    value = total_packets / dev_time
    e2e = total_packets / e2e_time
    steps_per_packet = tally.steps / n
    events_per_packet = tally.events / n
    trapped = tally.trapped
    clocks = clk.summary()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    prof = load_roofline_profile()
    roof = {"bound": "issue", "unit": "Gthread-inst/s", "achieved": None, "peak": None,
            "frac": None, "traffic": None,
            "note": "issue-rate roofline: SMs x SM clock x 128 lanes vs photon-steps/s x "
                    "thread-instructions per step (ncu, profiles/)"}
    steps_per_s = tally.steps * world * args.steps / dev_time
    if prof and clocks.get("sm_mhz") and st == "bench1":
        ips = float(prof["thread_inst_per_step"])
        peak = sms * clocks["sm_mhz"] * 1e6 * 128 / 1e9
        ach = steps_per_s * ips / 1e9
        roof.update(achieved=ach, peak=peak, frac=ach / peak,
                    traffic=prof.get("dram_bytes_per_launch"),
                    thread_inst_per_step=ips, steps_per_s=steps_per_s,
                    roofline_steps_per_s=peak * 1e9 / ips, clock="median SM clock under load",
                    source=os.path.relpath(ROOFLINE_FILE, ROOT))
        # frac counts issue slots, whatever share of a warp's 32 lanes each
        # instruction carries; these two count lanes that did work
        if prof.get("thread_inst_executed_per_step"):
            exe = float(prof["thread_inst_executed_per_step"])
            roof.update(active_lane_frac=exe / ips,
                        useful_frac=steps_per_s * exe / (peak * 1e9),
                        thread_inst_executed_per_step=exe,
                        useful_note="useful_frac = photon-steps/s x executed thread-instructions "
                                    "per step / (SMs x clock x 128): the issue-rate fraction "
                                    "with idle lanes of divergent instructions not counted")
        if prof.get("algorithmic_inst_per_step"):
            alg = float(prof["algorithmic_inst_per_step"])
            roof.update(algorithmic_frac=steps_per_s * alg / (peak * 1e9),
                        algorithmic_inst_per_step=alg,
                        algorithmic_note="the building blocks a photon-step needs (Philox block, "
                                         "spin, free path, its share of interface, incidence "
                                         "and sphere work), per ncu counts of each block alone")
    else:
        roof.update(steps_per_s=steps_per_s)
    # the HBM side, for completeness: DRAM bytes per launch (ncu) over the launch
    # time, against the measured copy bandwidth
    peaks = load_measured_peaks()
    if prof and prof.get("dram_bytes_per_launch") and peaks.get("hbm_gbs"):
        gbs = prof["dram_bytes_per_launch"] / (dev_time / args.steps) / 1e9
        roof["hbm"] = {"achieved_gbs": gbs, "peak_gbs": peaks["hbm_gbs"],
                       "frac": gbs / peaks["hbm_gbs"], "peak_source": "MEASURED_PEAKS.json (of measured)"}
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        # the reference's own Python where it was staged, with the FP64
        # restatement beside it; else the restatement
        port = cpu_baseline(stack=st)
        cpu = refpython_baseline(stack=st)
        if cpu is None:
            cpu = port
        else:
            cpu["port"] = port
    line = {"metric": "photons/s", "value": value, "unit": "photons/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dev_time / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": dict(workload_config(st, n), tune={"block_threads": int(tuned.block_threads),
                                                         "chunk": "sized on the device per batch"}),
            "e2e": {"value": e2e, "unit": "photons/s", "h2d_bytes_per_step": C.sizeof(_abi.Instance),
                    "d2h_bytes_per_step": C.sizeof(_abi.Tally),
                    "api": "ismc_run_batch (host pointers)"},
            "gpu_launches": 3 * args.steps,
            "clocks": clocks,
            "roofline": roof,
            "cpu_baseline": cpu,
            "result": {"R_d": res.mean[1], "T_d": res.mean[3], "T_u": res.mean[4],
                       "se": [res.se[1], res.se[3], res.se[4]], "packets": res.n,
                       "steps_per_packet": steps_per_packet, "events_per_packet": events_per_packet,
                       "trapped_packets": trapped}}
    if merge is not None:
        line["merge"] = merge
    print(json.dumps(line), flush=True)


def run_other_workload(args):
    """Secondary workloads of the benchmark set (one JSON line each); the
    default workload above is the headline line."""
    from ismc_gb300 import Engine, benchmarks, build
    build.build()
    eng = Engine(0)
    s = args.scale
    if args.workload == "dropin":
        run_dropin_workload()
        return
    if args.workload == "train":
        r = benchmarks.run_train(epochs=max(2, int(8 * s)))
        peaks = load_measured_peaks()
        peak = peaks.get("bf16_tflops")
        line = {"metric": "surrogate training steps/s", "value": r["steps_per_s"],
                "unit": "steps/s", "higher_is_better": True, "workload": "train",
                "dtype": "bf16 (fp32 accumulate)",
                "config": {"workload": "MLP 5-256-256-256-6, batch 4096, Gaussian NLL + Adam, "
                                       "device-resident synthetic rows", "scale": s},
                "roofline": {"bound": "tensor", "unit": "TFLOP/s", "achieved": r["tflops"],
                             "peak": peak, "frac": r["tflops"] / peak if peak else None,
                             "traffic": None,
                             "note": "algorithmic FLOP per step over host-timed steps (13 "
                                     "launches each); peak = measured bf16 burst "
                                     "(MEASURED_PEAKS.json, of measured)"},
                "result": r}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "tables":
        r, data = benchmarks.run_tables(eng, grid=max(8, int(64 * min(1.0, s))),
                                        N=max(50, int(1000 * min(1.0, s))), M=100)
        cpu = None if args.no_cpu_baseline else cpu_tables_baseline(data, N=r["N"], M=r["M"])
        line = {"metric": "lookup-table inversion time", "value": r["tables_s"], "unit": "s",
                "higher_is_better": False, "workload": "tables",
                "config": {"workload": "grid x grid single-slab lookup (1e5 packets x 4 runs), then "
                                       "makelookup: 4 Clough-Tocher N x N tables + M-draw "
                                       "uncertainty map", "scale": s},
                "cpu_baseline": cpu, "result": r}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "lookup":
        r = benchmarks.run_lookup(eng, scale=s)
        r["scale"] = s
        cpu = None if args.no_cpu_baseline else cpu_lookup_baseline(r)
        line = {"metric": "photons/s", "value": r["photons_per_s"], "unit": "photons/s",
                "workload": "lookup", "cpu_baseline": cpu, "config": {"workload": "64x64 single-slab grid + 512 random "
                "1-5 layer stacks, budgets log-uniform 1e5-1e7 x scale, one persistent launch",
                "scale": s}, "result": r}
    else:
        if args.load_surrogate:
            # a network trained and saved by an earlier run of this workload
            import numpy as np
            from ismc_gb300.surrogate import Surrogate
            sur = Surrogate(0, max_batch=4096, seed=42)
            sur.set_params(np.load(args.load_surrogate))
            r = {"loaded": args.load_surrogate}
        else:
            hg = args.heldout if args.heldout is not None else (32 if s >= 1 else 12)
            sur, r = benchmarks.run_surrogate(
                eng, n_samples=int((1 << 20) * s) // 4096 * 4096 or 4096,
                packets=max(1000, int(100_000 * min(1.0, s * 4))), epochs=args.epochs,
                heldout=hg, heldout_packets=10_000_000 if s >= 1 else 1_000_000)
        if args.save_surrogate:
            import numpy as np
            np.save(args.save_surrogate, sur.get_params())
        line = {"workload": "surrogate", "config": {"scale": s, "epochs": args.epochs},
                "result": r}
        if args.workload == "solve":
            sr = benchmarks.run_solve(eng, sur, n_meas=max(256, int(10000 * s)),
                                      n_plain=max(32, int(200 * min(1.0, 4 * s))))
            cpu = None if args.no_cpu_baseline else cpu_solve_baseline(eng)
            line = {"metric": "inverse solves/s", "value": sr["surrogate_solves_per_s"],
                    "cpu_baseline": cpu,
                    "unit": "solves/s", "workload": "solve",
                    "config": {"scale": s, "epochs": args.epochs},
                    "result": sr, "surrogate": r}
        sur.close()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--stack", choices=["bench1", "bench1_noslides", "bench0", "bench0_noslides"],
                    default="bench1", help="layer stack of the forward workload (default: the "
                                           "multilayer benchmark configuration)")
    ap.add_argument("--packets", type=int, default=PACKETS,
                    help="packets per step (the refpython arm sizes its steps itself unless "
                         "this is given)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["forward", "lookup", "tables", "surrogate", "solve",
                                           "dropin", "train", "refcuda", "refpython"],
                    default="forward")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="size factor for the secondary workloads (1 = full benchmark size)")
    ap.add_argument("--save-surrogate", default=None,
                    help="save the trained surrogate's parameters (.npy) here")
    ap.add_argument("--load-surrogate", default=None,
                    help="use saved surrogate parameters (.npy) instead of training")
    ap.add_argument("--heldout", type=int, default=None,
                    help="points per axis of the surrogate's held-out grid (default 32 at full "
                         "scale; each point is a 1e7-packet run)")
    ap.add_argument("--epochs", type=int, default=20,
                    help="training epochs of the surrogate (surrogate and solve workloads)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == "refcuda":
        if args.impl != "reference":
            ap.error("--workload refcuda is the reference CUDA arm: use --impl reference")
        run_refcuda(args, rank)
        return
    if args.workload == "refpython":
        if args.impl != "reference":
            ap.error("--workload refpython is a reference arm: use --impl reference")
        run_refpython(args, rank)
        return
    if args.workload != "forward":
        if rank == 0 and args.impl == "gpu":
            run_other_workload(args)
        return
    dist = None
    if world > 1:
        import torch.distributed as tdist
        backend = "gloo" if args.impl == "reference" else "nccl"
        tdist.init_process_group(backend)
        dist = tdist
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gpu(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
