"""The reference's own Python forward model, timed on the host cores.

ORACLE / baseline infrastructure only: bench.py's reference arm
(`--impl reference --workload refpython`) and tests/ use it; nothing in the
product does.

ISMLMC() (ISMLMC.py:101-347, with the walk of MLMC.py:283-409) is imported
from the unmodified copies that oracle/build_ref.py stages into
oracle/_ref/python/.  It is single-threaded pure Python, so the run spreads
packets over a `spawn` process pool: worker k seeds Python's `random` with
seed + k and simulates an equal share, as tests/golden/make_golden.py does.
The tallies come back as the reference returns them (fractions rounded to
len(str(N)) digits, ISMLMC.py:333-338) and are pooled as packet-weighted
means.
"""
import contextlib
import io
import multiprocessing as mp
import sys
import time


def _batch(args):
    """One worker's share: (A, R_d, R_s, T_d, T_u) of the reference's ISMLMC()
    and the CPU seconds it took.  Its two result printouts are discarded."""
    model_dir, layers, sph, n, seed = args
    if model_dir not in sys.path:
        sys.path.insert(0, model_dir)
    import random
    import ISMLMC
    random.seed(seed)
    nl = [L[0] for L in layers]
    mua = [L[1] for L in layers]
    mus = [L[2] for L in layers]
    g = [L[3] for L in layers]
    t = [L[4] for L in layers]
    mut = [a + s for a, s in zip(mua, mus)]
    s = sph
    t0 = time.process_time()
    with contextlib.redirect_stdout(io.StringIO()):
        out = ISMLMC.ISMLMC(n, nl, g, t, mua, mus, mut, s["R"], s["R_pw"], s["R_fs"], s["R_fp"],
                            s["R_fd"], s["R_f"], s["R_angle"], s["specular_included"], s["T"],
                            s["T_pw"], s["T_fs"], s["T_fp"], s["T_fd"], s["T_f"], s["T_angle"])
    return [float(v) for v in out], time.process_time() - t0


def layer_tuples(layers):
    """(n, mua, mus, g, d) per layer from ismc_gb300.Layer objects."""
    return [(float(L.n), float(L.mua), float(L.mus), float(L.g), float(L.d)) for L in layers]


def sphere_dict(sp):
    """The reference's sphere arguments from an ismc_gb300.Spheres."""
    keys = ("R", "R_pw", "R_fs", "R_fp", "R_fd", "R_f", "R_angle", "specular_included",
            "T", "T_pw", "T_fs", "T_fp", "T_fd", "T_f", "T_angle")
    return {k: getattr(sp, k) for k in keys}


def instance_args(inst):
    """(layer tuples, sphere arguments) of an ismc_gb300 ctypes instance."""
    st, sp = inst.stack, inst.spheres
    layers = [(float(st.n[l]), float(st.mua[l]), float(st.mus[l]), float(st.g[l]), float(st.d[l]))
              for l in range(int(st.L))]
    keys = ("R_pw", "R_fs", "R_fp", "R_fd", "R_f", "R_angle",
            "T_pw", "T_fs", "T_fp", "T_fd", "T_f", "T_angle")
    sph = {k: float(getattr(sp, k)) for k in keys}
    sph.update(R=bool(sp.R), T=bool(sp.T), specular_included=bool(sp.specular_included))
    return layers, sph


class Runner:
    """A pool of `procs` spawned workers running the staged reference model."""

    def __init__(self, model_dir, procs):
        self.model_dir = model_dir
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs)
        self.last_batches = []

    def run(self, layers, sph, packets_per_worker, seed):
        """All workers simulate `packets_per_worker` packets each (worker k
        seeded with seed + k).  Returns (pooled tallies, wall seconds, CPU
        seconds summed over workers).  The workers' own tallies are kept in
        self.last_batches."""
        jobs = [(self.model_dir, layers, sph, int(packets_per_worker), seed + k)
                for k in range(self.procs)]
        t0 = time.perf_counter()
        res = self.pool.map(_batch, jobs)
        wall = time.perf_counter() - t0
        self.last_batches = [r[0] for r in res]
        tallies = [sum(r[0][i] for r in res) / len(res) for i in range(5)]
        return tallies, wall, sum(r[1] for r in res)

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
