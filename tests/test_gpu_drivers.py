"""The reference's own driver scripts, unmodified, end to end on this engine.

Minimization/minimization.py and Lookup/lookup.py (byte-for-byte copies staged
by oracle/build_ref.py; the tests skip where none were staged) run through
ismc_gb300.dropin.drivers, which patches only removed Python / numpy APIs in
memory.  Their Python path calls the drop-in ISMC (the GPU propagator); their
CUDA path shells out to the drop-in programs ismc_gb300/bin/minimize.o and
Lookup.o.  Small configurations derived from the reference's example.ini keep
each run to seconds.  Each run must finish, print its answer in the reference's
format, and that answer must reproduce the measurement it was solved from: the
propagator at the printed (mu_a, mu_s') gives R_d and T_d within a few percent
of the configuration's M_R and M_T.
"""
import configparser
import os
import re
import shutil
import subprocess
import sys

import pytest

from ismc_gb300 import Engine, Layer, Spheres, make_instance

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _staged(rel):
    from oracle import build_ref
    return build_ref.staged_driver(rel)


def _need(rel):
    return pytest.mark.skipif(_staged(rel) is None, reason="reference drivers not staged")


def _copy(tmp, rel, edits, drop=()):
    """The staged driver and a copy of its example.ini with `edits`
    ({(section, key): value}) and without the keys `drop`, in a fresh directory."""
    sub = os.path.dirname(rel)
    d = tmp / sub
    d.mkdir()
    drv = d / os.path.basename(rel)
    shutil.copyfile(_staged(rel), drv)
    cp = configparser.ConfigParser()
    cp.read(_staged(os.path.join(sub, "example.ini")))
    for (sec, key), val in edits.items():
        cp.set(sec, key, str(val))
    for sec, key in drop:
        cp.remove_option(sec, key)
    ini = d / "small.ini"
    with open(ini, "w") as fh:
        cp.write(fh)
    return str(drv), str(ini), cp


def _run(drv, args, cwd, timeout=900):
    cmd = [sys.executable, "-m", "ismc_gb300.dropin.drivers", drv] + args
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r.stdout


def _reproduces(cp, mua, mus_r, tol):
    """R_d (R sphere only) and T_d (T sphere only) of the slab at (mua, mus'),
    as the driver's separate-sphere cost simulates them (minimization.py:208-217),
    against the configuration's M_R and M_T."""
    n, g, t = (float(cp.get("sample", k)) for k in ("n", "g", "t"))
    f = lambda k: float(cp.get("spheres", k))
    sph = dict(R_pw=f("R_pw"), R_fs=f("R_fs"), R_fp=f("R_fp"), R_fd=f("R_fd"),
               T_pw=f("T_pw"), T_fs=f("T_fs"), T_fp=f("T_fp"), T_fd=f("T_fd"))
    ly = [Layer.from_reduced(n, mua, mus_r, g, t)]
    with Engine(0) as eng:
        rd = eng.run_batch([make_instance(ly, Spheres(R=True, T=False, **sph), 400_000, seed=3,
                                          roulette_threshold=1e-3)])[0]["R_d"]
        td = eng.run_batch([make_instance(ly, Spheres(R=False, T=True, **sph), 400_000, seed=4,
                                          roulette_threshold=1e-3)])[0]["T_d"]
    m_r = float(cp.get("experiment", "M_R").split("\n")[0])
    m_t = float(cp.get("experiment", "M_T").split("\n")[0])
    assert abs(rd / m_r - 1) < tol and abs(td / m_t - 1) < tol, (mua, mus_r, rd, m_r, td, m_t)


_ANSWER = re.compile(r"mu_a: (\S+) \+/- (\S+) 1/cm\nmu_s': (\S+) \+/- (\S+) 1/cm")

# the example's sample and spheres with their uncertainties set to zero, so
# every uncertainty sample solves the same problem
_EXACT = {("sample", "n_unc"): 0.0, ("spheres", "R_pw_unc"): 0.0, ("spheres", "R_fs_unc"): 0.0,
          ("spheres", "R_fp_unc"): 0.0, ("spheres", "R_fd_unc"): 0.0,
          ("spheres", "T_pw_unc"): 0.0, ("spheres", "T_fs_unc"): 0.0,
          ("spheres", "T_fp_unc"): 0.0, ("spheres", "T_fd_unc"): 0.0,
          ("spheres", "T_angle_unc"): 0.0}
# fewer repetitions, a start nearer the answer, and only the two measurements
# the answer is checked against: the example's unscattered transmittance is
# fitted against an angle given in degrees that the cost's ISMC() call reads
# as radians (minimization.py:218-220), which pulls its minimum off them
_MIN_EDITS = {**_EXACT, ("minimization", "N"): 100000, ("minimization", "runs"): 1,
              ("minimization", "input_distributions_samples"): 2,
              ("minimization", "mua_guess"): 2.0, ("minimization", "mus_guess"): 30.0,
              ("minimization", "tolerance"): 0.01}
_MIN_DROP = (("experiment", "M_U"), ("experiment", "M_U_unc"))


@_need("Minimization/minimization.py")
def test_minimization_driver_python_path(tmp_path):
    """minimization.py --Python: scipy Powell over the drop-in ISMC, seeded, so
    two runs print the same answer, and that answer fits the measurement."""
    drv, ini, cp = _copy(tmp_path, "Minimization/minimization.py", _MIN_EDITS, _MIN_DROP)
    args = ["--numpy-seed", "5", "--ismc-seed", "7", "--Python", ini]
    out1 = _run(drv, args, os.path.dirname(drv))
    out2 = _run(drv, args, os.path.dirname(drv))
    m1, m2 = _ANSWER.search(out1), _ANSWER.search(out2)
    assert m1 and m2, out1[-2000:]
    assert m1.groups() == m2.groups()
    _reproduces(cp, float(m1.group(1)), float(m1.group(3)), 0.05)


@_need("Minimization/minimization.py")
def test_minimization_driver_cuda_path(tmp_path):
    """minimization.py --CUDA: the driver builds minimize.o command lines
    (minimization.py:169-196) and parses its four numbers."""
    from ismc_gb300 import build
    build.build()
    drv, ini, cp = _copy(tmp_path, "Minimization/minimization.py", _MIN_EDITS, _MIN_DROP)
    exe = os.path.join(ROOT, "ismc_gb300", "bin", "minimize.o")
    out = _run(drv, ["--numpy-seed", "5", "--CUDA", "--CUDAsource", exe, "--GPU", "0", ini],
               os.path.dirname(drv))
    m = _ANSWER.search(out)
    assert m, out[-2000:]
    _reproduces(cp, float(m.group(1)), float(m.group(3)), 0.05)


@_need("Lookup/lookup.py")
def test_lookup_driver_cuda_path_gpu_tables(tmp_path):
    """lookup.py --CUDA with the GPU tables: Lookup.o generates the grid, the
    GPU makelookup builds the cubic tables and the uncertainty map, and the
    driver's own lookup of the example measurement must fit it."""
    from ismc_gb300 import build
    build.build()
    edits = {**_EXACT, ("lookup", "N"): 50000, ("lookup", "runs"): 2,
             ("lookup", "dimensions"): 300, ("lookup", "simulation_distributions_samples"): 20,
             ("lookup", "measurement_distributions_samples"): 100,
             ("lookup", "input_distributions_samples"): 2}
    drv, ini, cp = _copy(tmp_path, "Lookup/lookup.py", edits)
    exe = os.path.join(ROOT, "ismc_gb300", "bin", "Lookup.o")
    # lookup.py's --GPU takes a list (nargs="*"): the configuration file goes first
    out = _run(drv, ["--gpu-tables", "--numpy-seed", "5", "--CUDA", "--CUDAsource", exe, ini,
                     "--GPU", "0"], os.path.dirname(drv))
    ma = re.search(r"mua = (\S+) \+/- (\S+) for R_d", out)
    ms = re.search(r"mus' = (\S+) \+/- (\S+) for R_d", out)
    assert ma and ms, out[-2000:]
    prefix = cp.get("lookup", "filename_prefix")
    tables = os.path.join(os.path.dirname(drv), f"{prefix}_lookup_tables")
    assert os.path.exists(tables + ".npz") or os.path.exists(tables + ".h5")
    # the table is 300 x 300 over 0-100 % in R and T: lookups resolve ~0.3 %
    _reproduces(cp, float(ma.group(1)), float(ms.group(1)), 0.08)


@_need("Lookup/lookup.py")
def test_lookup_driver_python_path_gpu_tables(tmp_path):
    """lookup.py --Python with the GPU tables: the reference's own
    sample_space loop (lookup.py:228-259) calls the drop-in ISMC for every
    grid point, run and input sample; the GPU makelookup builds the tables,
    and the driver's own lookup of the example measurement must fit it."""
    edits = {**_EXACT, ("lookup", "N"): 50000, ("lookup", "runs"): 2,
             ("lookup", "dimensions"): 300, ("lookup", "simulation_distributions_samples"): 20,
             ("lookup", "measurement_distributions_samples"): 100,
             ("lookup", "input_distributions_samples"): 2}
    drv, ini, cp = _copy(tmp_path, "Lookup/lookup.py", edits)
    out = _run(drv, ["--gpu-tables", "--numpy-seed", "5", "--ismc-seed", "7", "--Python", ini],
               os.path.dirname(drv))
    ma = re.search(r"mua = (\S+) \+/- (\S+) for R_d", out)
    ms = re.search(r"mus' = (\S+) \+/- (\S+) for R_d", out)
    assert ma and ms, out[-2000:]
    assert out.count("RUN: ") == 13 * 11 * 2 * 2          # grid x runs x input samples
    _reproduces(cp, float(ma.group(1)), float(ms.group(1)), 0.08)


@_need("Lookup/lookup.py")
def test_lookup_driver_python_path_reference_tables(tmp_path):
    """lookup.py --Python without the GPU tables: the driver's own
    makelookup (scipy griddata and its Python uncertainty loop,
    lookup.py:301-465) turns the drop-in ISMC grid into the tables, at a
    150 x 150 resolution to keep its loop short."""
    edits = {**_EXACT, ("lookup", "N"): 50000, ("lookup", "runs"): 2,
             ("lookup", "dimensions"): 150, ("lookup", "simulation_distributions_samples"): 20,
             ("lookup", "measurement_distributions_samples"): 100,
             ("lookup", "input_distributions_samples"): 2}
    drv, ini, cp = _copy(tmp_path, "Lookup/lookup.py", edits)
    out = _run(drv, ["--numpy-seed", "5", "--ismc-seed", "7", "--Python", ini],
               os.path.dirname(drv))
    ma = re.search(r"mua = (\S+) \+/- (\S+) for R_d", out)
    ms = re.search(r"mus' = (\S+) \+/- (\S+) for R_d", out)
    assert ma and ms, out[-2000:]
    # a 150 x 150 table over 0-100 % in R and T resolves ~0.7 %
    _reproduces(cp, float(ma.group(1)), float(ms.group(1)), 0.10)
