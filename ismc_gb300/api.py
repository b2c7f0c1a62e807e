"""Python host API over the C ABI (include/ismc.h).

This is the layer the reference's callers reach through the drop-in modules
(``ismc_gb300.dropin.ISMC`` / ``ISMLMC``) and the batch drivers.  It builds the
ABI structs, calls ``libismc.so`` and turns integer tallies into FP64 means and
standard errors.  There is no CPU fallback: without the CUDA library or a GPU
every call raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import threading
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

from . import _abi

_LIB = None
_LIB_LOCK = threading.Lock()
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libismc.so")


class IsmcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ismc error {code} ({_abi.ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


def load_library(path: str = LIB_PATH):
    """Load and check libismc.so (built in-tree by ``python -m ismc_gb300.build``)."""
    global _LIB
    with _LIB_LOCK:
        if _LIB is None:
            if not os.path.exists(path):
                raise RuntimeError(f"{path} is missing: build it with `python -m ismc_gb300.build`"
                                   " (the GPU path has no CPU fallback)")
            _LIB = _abi.declare(C.CDLL(path))
        return _LIB


# ----------------------------------------------------------------------------
# inputs
# ----------------------------------------------------------------------------
@dataclass
class Layer:
    """One layer: refractive index, absorption and scattering coefficients (1/cm),
    anisotropy g and thickness d (cm).  mus == 0 marks a non-scattering slide.
    mut defaults to mua + mus, as the reference's callers pass it
    (lookup.py:238, minimization.py:205)."""
    n: float
    mua: float
    mus: float
    g: float
    d: float
    mut: Optional[float] = None

    @staticmethod
    def slide(n=1.5, d=0.1):
        return Layer(n, 0.0, 0.0, 0.0, d)

    @staticmethod
    def from_reduced(n, mua, mus_reduced, g, d):
        """mu_s from the reduced coefficient: mu_s = mu_s' / (1 - g), or mu_s' when g == 1
        (ISMC.py:28-29)."""
        mus = mus_reduced if g == 1 else mus_reduced / (1.0 - g)
        return Layer(n, mua, mus, g, d)


def cap_fraction(port_radius, sphere_radius):
    """Area fraction of a circular port on a sphere (spherical cap):
    f = (1 - sqrt(1 - (a/Rs)^2)) / 2."""
    return 0.5 * (1.0 - math.sqrt(1.0 - (port_radius / sphere_radius) ** 2))


@dataclass
class Spheres:
    """Two-sphere geometry with the reference's argument meaning (ISMC.py:34-50).
    Angles in radians."""
    R: bool = True
    R_pw: float = 0.99
    R_fs: float = 0.02351
    R_fp: float = 0.054638
    R_fd: float = 0.02351
    R_f: Optional[float] = None
    R_angle: float = math.pi / 10
    specular_included: bool = False
    T: bool = False
    T_pw: float = 0.99
    T_fs: float = 0.054638
    T_fp: float = 0.02351
    T_fd: float = 0.02351
    T_f: Optional[float] = None
    T_angle: float = 0.22 * math.pi / 180

    def __post_init__(self):
        if self.R_f is None:
            self.R_f = self.R_fs + self.R_fp + self.R_fd
        if self.T_f is None:
            self.T_f = self.T_fs + self.T_fp + self.T_fd

    @staticmethod
    def from_radii(sphere_radius=5.08, sample_port=1.27, entrance_port=1.27, detector_port=0.635,
                   wall=0.98, R=True, T=True, specular_included=False,
                   R_angle=math.pi / 10, T_angle=0.22 * math.pi / 180):
        """Port radii (cm) -> the reference's area fractions; the T sphere's
        optional port takes the entrance-port size."""
        fs = cap_fraction(sample_port, sphere_radius)
        fp = cap_fraction(entrance_port, sphere_radius)
        fd = cap_fraction(detector_port, sphere_radius)
        return Spheres(R=R, R_pw=wall, R_fs=fs, R_fp=fp, R_fd=fd, R_angle=R_angle,
                       specular_included=specular_included, T=T, T_pw=wall, T_fs=fs, T_fp=fp,
                       T_fd=fd, T_angle=T_angle)


def make_stack(layers: Sequence[Layer]) -> _abi.Stack:
    if not 1 <= len(layers) <= _abi.MAXL:
        raise ValueError(f"a stack has 1..{_abi.MAXL} layers, got {len(layers)}")
    s = _abi.Stack()
    s.L = len(layers)
    for i, ly in enumerate(layers):
        s.n[i] = ly.n
        s.mua[i] = ly.mua
        s.mus[i] = ly.mus
        s.mut[i] = ly.mua + ly.mus if ly.mut is None else ly.mut
        s.g[i] = ly.g
        s.d[i] = ly.d
    return s


def make_spheres(sp: Spheres) -> _abi.Spheres:
    x = _abi.Spheres()
    x.R = 1 if sp.R else 0
    x.T = 1 if sp.T else 0
    x.specular_included = 1 if sp.specular_included else 0
    for k in ("R_pw", "R_fs", "R_fp", "R_fd", "R_f", "R_angle",
              "T_pw", "T_fs", "T_fp", "T_fd", "T_f", "T_angle"):
        setattr(x, k, float(getattr(sp, k)))
    return x


MODES = {"compat": _abi.MODE_COMPAT, "physical": _abi.MODE_PHYSICAL,
         _abi.MODE_COMPAT: _abi.MODE_COMPAT, _abi.MODE_PHYSICAL: _abi.MODE_PHYSICAL}


def make_instance(layers: Sequence[Layer], spheres: Spheres, n_packets: int, seed: int = 0,
                  stream: int = 0, mode="compat", roulette_threshold: float = 1e-4,
                  roulette_m: float = 10.0, packet_offset: int = 0) -> _abi.Instance:
    """One simulation instance.  roulette_threshold 1e-4 / m = 10 are MLMC.py:86-87;
    the single-slab driver of ISMC.py:136 uses 1e-3."""
    inst = _abi.Instance()
    inst.stack = make_stack(layers)
    inst.spheres = make_spheres(spheres)
    inst.n_packets = int(n_packets)
    inst.packet_offset = int(packet_offset)
    inst.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    inst.stream = int(stream) & 0xFFFFFFFF
    inst.mode = MODES[mode]
    inst.roulette_threshold = roulette_threshold
    inst.roulette_m = roulette_m
    return inst


def instance_array(instances: Sequence[_abi.Instance]):
    arr = (_abi.Instance * len(instances))()
    for i, x in enumerate(instances):
        arr[i] = x
    return arr


# ----------------------------------------------------------------------------
# outputs
# ----------------------------------------------------------------------------
@dataclass
class Result:
    """Normalised outcome of one instance: fractions of N as the reference
    returns them (ISMC.py:406), their standard errors, and counters."""
    n: int
    mean: List[float]
    se: List[float]
    status: int
    steps: int
    events: int
    reincidences: int
    capped: int
    trapped: int
    analytic_specular: float
    analytic_ballistic: float
    sums: List[int] = field(repr=False, default_factory=list)
    sumsqs: List[int] = field(repr=False, default_factory=list)

    def as_tuple(self):
        return tuple(self.mean)

    def __getitem__(self, name):
        return self.mean[_abi.TALLIES.index(name)]


def tally_to_result(t: _abi.Tally) -> Result:
    """FP64 normalisation of the fixed-point sums: mean = S/(N 2^k),
    SE = sqrt((Q/(N 2^k) - mean^2) / (N - 1))."""
    return merge_tallies([t])


def merge_tallies(tallies) -> Result:
    """One Result from the tallies of consecutive packet ranges of one
    simulation (split_instance): the integer sums add exactly (Python
    integers, so beyond 64 bits too), statuses combine by minimum (any error
    wins), and the normalisation is tally_to_result's."""
    t0 = tallies[0]
    n = sum(int(t.n) for t in tallies)
    sums = [sum(int(t.sum[k]) for t in tallies) for k in range(5)]
    sumsqs = [sum(int(t.sumsq[k]) for t in tallies) for k in range(5)]
    scale = float(2 ** int(t0.scale_log2 or 32))
    mean, se = [], []
    for k in range(5):
        s, q = sums[k], sumsqs[k]
        if n > 0:
            m = s / scale / n
            ex2 = q / scale / n
            var = max(ex2 - m * m, 0.0) * n / (n - 1) if n > 1 else 0.0
            mean.append(m)
            se.append(math.sqrt(var / n))
        else:
            mean.append(float("nan"))
            se.append(float("nan"))
    total = lambda f: sum(int(getattr(t, f)) for t in tallies)
    return Result(n=n, mean=mean, se=se, status=min(int(t.status) for t in tallies),
                  steps=total("steps"), events=total("events"),
                  reincidences=total("reincidences"), capped=total("capped"),
                  trapped=total("trapped"), analytic_specular=float(t0.analytic_specular),
                  analytic_ballistic=float(t0.analytic_ballistic), sums=sums, sumsqs=sumsqs)


def split_instance(inst: _abi.Instance, max_packets: int = _abi.MAX_PACKETS):
    """An instance as consecutive packet ranges of at most max_packets each.
    Every draw is keyed by the packet id, so the parts' summed tallies equal
    one run of the whole range (ISMC_MAX_PACKETS bounds one instance)."""
    n = int(inst.n_packets)
    if n <= max_packets:
        return [inst]
    parts = []
    for lo in range(0, n, max_packets):
        x = _abi.Instance.from_buffer_copy(bytes(inst))
        x.packet_offset = int(inst.packet_offset) + lo
        x.n_packets = min(max_packets, n - lo)
        parts.append(x)
    return parts


def tallies_mean_se(tallies):
    """Vectorised tally_to_result for a ctypes array of tallies: (mean [n x 5],
    se [n x 5], status [n]) with the same FP64 normalisation."""
    import numpy as np
    v = np.ctypeslib.as_array(tallies)
    n = v["n"].astype(np.float64)
    scale = np.ldexp(1.0, np.where(v["scale_log2"] == 0, 32, v["scale_log2"]).astype(np.int64))
    s = v["sum"].astype(np.float64) / scale[:, None]
    q = v["sumsq"].astype(np.float64) / scale[:, None]
    with np.errstate(invalid="ignore", divide="ignore"):
        mean = s / n[:, None]
        ex2 = q / n[:, None]
        var = np.where(n[:, None] > 1, np.maximum(ex2 - mean * mean, 0.0) * n[:, None] /
                       np.maximum(n[:, None] - 1, 1), 0.0)
        se = np.sqrt(var / n[:, None])
    bad = n == 0
    mean[bad] = np.nan
    se[bad] = np.nan
    return mean, se, v["status"].copy()


def slab_instances(mua, mus_reduced, g, d, n, spheres: Spheres, n_packets, seed: int = 0,
                   stream0: int = 0, mode="compat", slides=((1.5, 0.1), (1.5, 0.1)),
                   roulette_threshold: float = 1e-4, roulette_m: float = 10.0):
    """Many one-slab instances between two slides at once: row i is
    make_instance([Layer.slide(*slides[0]), Layer.from_reduced(n[i], mua[i],
    mus_reduced[i], g[i], d[i]), Layer.slide(*slides[1])], spheres, n_packets,
    seed, stream0 + i, mode), filled as a numpy view of the ctypes array."""
    import numpy as np
    mua, musr, g, d, n = (np.atleast_1d(np.asarray(x, dtype=np.float64)) for x in
                          (mua, mus_reduced, g, d, n))
    m = max(len(mua), len(musr), len(g), len(d), len(n))
    mua, musr, g, d, n = (np.broadcast_to(x, (m,)) for x in (mua, musr, g, d, n))
    mus = np.where(g == 1.0, musr, musr / np.where(g == 1.0, 2.0, 1.0 - g))
    arr = (_abi.Instance * m)()
    v = np.ctypeslib.as_array(arr)
    st = v["stack"]
    st["L"] = 3
    (n0, d0), (n2, d2) = slides
    st["n"][:, 0], st["d"][:, 0] = n0, d0
    st["n"][:, 2], st["d"][:, 2] = n2, d2
    st["n"][:, 1] = n
    st["mua"][:, 1] = mua
    st["mus"][:, 1] = mus
    st["mut"][:, 1] = mua + mus
    st["g"][:, 1] = g
    st["d"][:, 1] = d
    sp = make_spheres(spheres)
    for name, _ in _abi.Spheres._fields_:
        v["spheres"][name] = getattr(sp, name) if not name.startswith("_") else 0
    v["n_packets"] = int(n_packets)
    v["packet_offset"] = 0
    v["seed"] = int(seed) & 0xFFFFFFFFFFFFFFFF
    v["stream"] = (np.arange(m, dtype=np.uint64) + np.uint64(stream0)) & np.uint64(0xFFFFFFFF)
    v["mode"] = MODES[mode]
    v["roulette_threshold"] = roulette_threshold
    v["roulette_m"] = roulette_m
    return arr


def make_solve(layers: Sequence[Layer], layer: int, spheres: Spheres, n_packets: int,
               meas, x0, lo=(1e-6, 1e-6), hi=(1e6, 1e6), seed: int = 0, separate=False,
               log_coords=True, h0=None, t0=None, max_evals=400, max_restarts=3,
               mode="compat", roulette_threshold=1e-4, fresh_streams=False,
               max_refits=2) -> _abi.SolveReq:
    """One plain-path inverse problem: find (mu_a, mu_s') of `layer` so that the
    simulated (R_d, R_s, T_d, T_u) match `meas` (None = not measured) under the
    reference's cost (minimization.py:231-238).  In log coordinates the PRAXIS
    step/tolerance default to 0.5 / 1e-3 (relative), else to the reference's
    example values 5 / 0.1 (Minimization/example.ini [minimization]).
    fresh_streams=False gives every evaluation of one solve the same Philox
    stream (common random numbers: the objective is then a deterministic
    function of the parameters); True draws a new stream per evaluation, as the
    reference's global random state does.  max_refits: how many times a
    minimisation that ended far above the objective's Monte Carlo noise is run
    again from where it ended (ismc_solve_req.max_refits)."""
    r = _abi.SolveReq()
    r.base = make_instance(layers, spheres, n_packets, seed=seed, mode=mode,
                           roulette_threshold=roulette_threshold)
    r.layer = int(layer)
    r.separate = 1 if separate else 0
    r.log_coords = 1 if log_coords else 0
    r.max_evals = int(max_evals)
    r.max_restarts = int(max_restarts)
    r.fresh_streams = 1 if fresh_streams else 0
    r.max_refits = int(max_refits)
    for k in range(4):
        r.meas[k] = float("nan") if meas[k] is None else float(meas[k])
    r.x0[0], r.x0[1] = float(x0[0]), float(x0[1])
    r.lo[0], r.lo[1] = float(lo[0]), float(lo[1])
    r.hi[0], r.hi[1] = float(hi[0]), float(hi[1])
    r.h0 = float(h0 if h0 is not None else (0.5 if log_coords else 5.0))
    r.t0 = float(t0 if t0 is not None else (1e-3 if log_coords else 0.1))
    return r


def make_tune(block_threads=0, blocks_per_sm=0, chunk_packets=0, max_events=0):
    return _abi.Tune(block_threads, blocks_per_sm, chunk_packets, max_events)


# ----------------------------------------------------------------------------
# engine
# ----------------------------------------------------------------------------
class Engine:
    """A propagator context on one GPU (wraps ismc_init / ismc_destroy).

    Not thread-safe: use one Engine per thread (or lock around it), as for the
    C context."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.ismc_init(int(device), C.byref(h))
        if rc != 0:
            raise IsmcError(rc, self._err(None))
        self.h = h
        self.device = device

    def _err(self, h):
        buf = C.create_string_buffer(1024)
        self.lib.ismc_last_error(h, buf, 1024)
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc != 0:
            raise IsmcError(rc, self._err(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ismc_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- single instance: ismc_run (MLMC.py roulette 1e-4 / m 10)
    def run(self, layers: Sequence[Layer], spheres: Spheres, n_packets: int, seed: int = 0,
            mode="compat") -> Result:
        if int(n_packets) > _abi.MAX_PACKETS:
            # the instance ismc_run builds, in parts of at most ISMC_MAX_PACKETS
            return self.run_batch([make_instance(layers, spheres, n_packets, seed=seed,
                                                 mode=mode)])[0]
        st = make_stack(layers)
        sp = make_spheres(spheres)
        out = _abi.Tally()
        rc = self.lib.ismc_run(self.h, C.byref(st), C.byref(sp), int(n_packets), int(seed),
                               MODES[mode], C.byref(out))
        if rc not in (0, _abi.ERR_STEP_LIMIT):
            self._check(rc)
        return tally_to_result(out)

    # -- many instances in one persistent launch: ismc_run_batch
    def run_batch_raw(self, instances, tune: Optional[_abi.Tune] = None):
        arr = instances if isinstance(instances, C.Array) else instance_array(instances)
        n = len(arr)
        out = (_abi.Tally * n)()
        rc = self.lib.ismc_run_batch(self.h, arr, n, C.byref(tune) if tune else None, out)
        self._check(rc)
        return out

    def run_batch(self, instances, tune: Optional[_abi.Tune] = None,
                  max_packets: int = _abi.MAX_PACKETS) -> List[Result]:
        """Results of a batch in one launch.  An instance of more than
        max_packets packets (at most ISMC_MAX_PACKETS, the C ABI's limit) runs
        as consecutive packet ranges in the same launch, merged exactly."""
        insts = list(instances)
        if all(int(x.n_packets) <= max_packets for x in insts):
            return [tally_to_result(t) for t in self.run_batch_raw(instances, tune)]
        parts, owner = [], []
        for i, x in enumerate(insts):
            for p in split_instance(x, max_packets):
                parts.append(p)
                owner.append(i)
        groups = [[] for _ in insts]
        for t, i in zip(self.run_batch_raw(parts, tune), owner):
            groups[i].append(t)
        return [merge_tallies(g) for g in groups]

    def run_batch_device(self, d_inst_ptr: int, n_inst: int, d_out_ptr: int, stream_ptr: int = 0,
                         tune: Optional[_abi.Tune] = None):
        """Enqueue a batch whose instances already live on the GPU (device pointers,
        e.g. torch uint8 tensors' data_ptr()); asynchronous on `stream_ptr`."""
        rc = self.lib.ismc_run_batch_device(self.h, C.c_void_p(d_inst_ptr), int(n_inst),
                                            C.byref(tune) if tune else None,
                                            C.c_void_p(d_out_ptr), C.c_void_p(stream_ptr))
        self._check(rc)

    def solve_batch(self, requests) -> List[_abi.SolveOut]:
        """Batched plain-path inverse solves (ismc_solve_batch): every round of
        objective evaluations of all active solves is one GPU launch."""
        arr = requests if isinstance(requests, C.Array) else (_abi.SolveReq * len(requests))(*requests)
        out = (_abi.SolveOut * len(arr))()
        self._check(self.lib.ismc_solve_batch(self.h, arr, len(arr), out))
        return list(out)

    def autotune(self, instances) -> _abi.Tune:
        arr = instances if isinstance(instances, C.Array) else instance_array(instances)
        t = _abi.Tune()
        self._check(self.lib.ismc_autotune(self.h, arr, len(arr), C.byref(t)))
        return t


_DEFAULT = {}


def default_engine(device: Optional[int] = None) -> Engine:
    """Process-wide engine per device (device from ISMC_DEVICE, default 0)."""
    dev = int(os.environ.get("ISMC_DEVICE", "0")) if device is None else int(device)
    key = (dev, threading.get_ident())
    if key not in _DEFAULT:
        _DEFAULT[key] = Engine(dev)
    return _DEFAULT[key]
