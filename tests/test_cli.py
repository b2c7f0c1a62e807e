"""The drop-in programs Lookup.o and minimize.o (ismc_gb300/bin/): flag
handling and exit codes as the reference's CUDA/ISMLMC-lookup.cu and
CUDA/ISMLMC-minimization.cu have them, the Diffuse_*.csv layout that
Lookup/lookup.py:188-214 parses, and the four-number stdout protocol that
Minimization/minimization.py:186-196 parses."""
import math
import os
import subprocess

import numpy as np
import pytest

from ismc_gb300 import build

BIN = os.path.join(os.path.dirname(build.__file__), "bin")


@pytest.fixture(scope="module")
def programs():
    build.build()
    return os.path.join(BIN, "Lookup.o"), os.path.join(BIN, "minimize.o")


def _run(cmd, cwd=None, timeout=600):
    return subprocess.run(cmd, capture_output=True, text=True, cwd=cwd, timeout=timeout)


def test_exit_codes_without_gpu_work(programs):
    lookup, minimize = programs
    assert _run([lookup, "--help"]).returncode == 1
    assert _run([minimize, "-h"]).returncode == 1
    r = _run([lookup, "-N", "10"])
    assert r.returncode == 2 and "--GPU" in r.stdout
    assert _run([minimize, "--runs", "2"]).returncode == 2
    # -N without --runs, and -N together with --unc, are rejected before any GPU work
    r = _run([lookup, "--GPU", "0", "-N", "1000", "--go"])
    assert r.returncode == 2 and "conjuction" in r.stdout
    r = _run([lookup, "--GPU", "0", "-N", "1000", "--runs", "2", "--unc", "0.01", "--go"])
    assert r.returncode == 2 and "cannot be used" in r.stdout


def _read_like_lookup_py(path, rows):
    """Parse a Diffuse_*.csv the way Lookup/lookup.py:188-214 does (np.float there
    is float here): averages, then the standard-error block."""
    data = np.genfromtxt(path, dtype=None, encoding=None, delimiter=",", invalid_raise=False)[2:, 2:]
    x, y = data.shape
    out = np.empty((x, y), dtype=object)
    for i in range(x):
        for j in range(y):
            try:
                out[i, j] = float(data[i, j].replace('"', ""))
            except ValueError:
                out[i, j] = data[i, j]
    out = np.delete(out, rows, 0)
    avg = out[0:rows, :].astype(float)
    se = out[rows + 1:, :].astype(float)
    return avg, se


@pytest.mark.gpu
def test_lookup_program_matches_batched_engine(programs, tmp_path):
    """A 3 x 4 table with two runs and separate spheres: the CSVs hold the
    float averages of the engine's tallies for the same instances, digit for digit."""
    from ismc_gb300 import _abi, api
    lookup, _ = programs
    Na, Ns, runs, N, seed = 3, 4, 2, 20000, 99
    n, g, t = 1.4, 0.5, 0.135
    sph_r = "0.99 0.02351 0.054638 0.02351"
    sph_t = "0.99 0.054638 0.02351 0.02351"
    cmd = [lookup, "--GPU", "0", "-N", str(N), "--runs", str(runs), "-n", str(n), "-g", str(g),
           "-t", str(t), "--Nmua", str(Na), "--muaS", "0.5", "--muaB", "1.5", "--Nmus", str(Ns),
           "--musS", "10", "--musB", "1.3", "--Rsphere", sph_r, "--Tsphere", sph_t,
           "--Tangle", "0.22", "--separate", "--go", "--seed", str(seed)]
    r = _run(cmd, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    Rm, Rse = _read_like_lookup_py(tmp_path / "Diffuse_Reflectance.csv", Na)
    Tm, Tse = _read_like_lookup_py(tmp_path / "Diffuse_Transmittance.csv", Na)
    assert Rm.shape == (Na, Ns) and Rse.shape == (Na, Ns)

    f32 = np.float32
    # float start * pow(double(float base), i) in double, stored as float
    mua = [f32(float(f32(0.5)) * math.pow(float(f32(1.5)), i)) for i in range(Na)]
    mus_ = [f32(float(f32(10)) * math.pow(float(f32(1.3)), j)) for j in range(Ns)]
    rp = [float(f32(v)) for v in sph_r.split()]
    tp = [float(f32(v)) for v in sph_t.split()]
    insts = []
    for _ in range(runs):
        for i in range(Na):
            for j in range(Ns):
                for k in range(2):
                    x = _abi.Instance()
                    x.stack.L = 1
                    x.stack.n[0], x.stack.g[0], x.stack.d[0] = f32(n), f32(g), f32(t)
                    x.stack.mua[0] = mua[i]
                    x.stack.mus[0] = f32(mus_[j] / (f32(1) - f32(g)))
                    x.stack.mut[0] = f32(x.stack.mua[0]) + f32(x.stack.mus[0])
                    s = x.spheres
                    s.R, s.T = (1, 0) if k == 0 else (0, 1)
                    if k == 0:
                        s.R_pw, s.R_fs, s.R_fp, s.R_fd = rp
                        s.R_f = float(f32(rp[1]) + f32(rp[2]) + f32(rp[3]))
                    else:
                        s.T_pw, s.T_fs, s.T_fp, s.T_fd = tp
                        s.T_f = float(f32(tp[1]) + f32(tp[2]) + f32(tp[3]))
                    s.T_angle = float(f32(float(f32(0.22)) * math.pi / 180))
                    x.n_packets, x.seed, x.stream = N, seed, len(insts)
                    x.mode, x.roulette_threshold, x.roulette_m = 0, 1e-4, 10.0
                    insts.append(x)
    eng = api.Engine(0)
    try:
        res = [api.tally_to_result(tt) for tt in eng.run_batch_raw(insts)]
    finally:
        eng.close()
    rd = np.array([f32(res[2 * q].mean[1]) for q in range(runs * Na * Ns)]).reshape(runs, Na, Ns)
    td = np.array([f32(res[2 * q + 1].mean[3]) for q in range(runs * Na * Ns)]).reshape(runs, Na, Ns)
    avg_r = (rd / f32(runs)).sum(0, dtype=np.float32)
    avg_t = (td / f32(runs)).sum(0, dtype=np.float32)
    fmt = np.vectorize(lambda v: float("%g" % float(v)))
    np.testing.assert_array_equal(Rm, fmt(avg_r))
    np.testing.assert_array_equal(Tm, fmt(avg_t))
    # standard errors: population sd / sqrt(runs), printed to 6 digits
    se_r = np.sqrt(((rd - avg_r) ** 2).sum(0) / runs) / math.sqrt(runs)
    np.testing.assert_allclose(Rse, se_r, rtol=1e-4, atol=1e-7)


@pytest.mark.gpu
def test_minimize_program_stdout_protocol(programs):
    """Measurements simulated at known (mu_a, mu_s') are recovered; the output is
    exactly four numbers as minimization.py reads them."""
    from ismc_gb300 import api
    _, minimize = programs
    n, g, t, mua, mus_ = 1.4, 0.5, 0.135, 1.5, 30.0
    sph = api.Spheres(R=True, R_pw=0.99, R_fs=0.02351, R_fp=0.054638, R_fd=0.02351,
                      T=True, T_pw=0.99, T_fs=0.054638, T_fp=0.02351, T_fd=0.02351)
    eng = api.Engine(0)
    try:
        truth = eng.run([api.Layer(n, mua, mus_ / (1 - g), g, t)], sph, 4_000_000, seed=5)
    finally:
        eng.close()
    cmd = [minimize, "--GPU", "0", "-N", "100000", "--runs", "4", "--step", "5", "--tol", "0.1",
           "-n", str(n), "-g", str(g), "-t", str(t), "--Rangle", "0", "--Tangle", "0",
           "--Rsphere", "0.99 0.02351 0.054638 0.02351", "--Tsphere", "0.99 0.054638 0.02351 0.02351",
           "--mua", "3", "--mus", "20", "--muaMin", "0.1", "--muaMax", "10", "--musMin", "1",
           "--musMax", "100", "--Rd", "%f" % truth.mean[1], "--Td", "%f" % truth.mean[3],
           "--go", "--seed", "3", "--crn"]
    r = _run(cmd)
    assert r.returncode == 0, r.stdout + r.stderr
    tok = [x for x in r.stdout.replace("\n", " ").split(" ") if x not in ("", "\n")]
    assert len(tok) == 4, r.stdout
    mua_hat, mua_se, mus_hat, mus_se = (float(x) for x in tok)
    assert abs(mua_hat / mua - 1) < 0.1, tok
    assert abs(mus_hat / mus_ - 1) < 0.05, tok
    assert mua_se >= 0 and mus_se >= 0


@pytest.mark.gpu
def test_minimize_program_reference_example(programs):
    """The reference's own example configuration (--example: initial guess
    (5, 45) outside its accepted box [1, 3] x [20, 40], separate spheres,
    1e4 packets per objective, 5 runs) completes with an answer in the box."""
    _, minimize = programs
    r = _run([minimize, "--GPU", "0", "--example", "--go", "--seed", "11"])
    assert r.returncode == 0, r.stdout + r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("mua:")]
    assert line, r.stdout
    mua = float(line[0].split()[1])
    mus = float([l for l in r.stdout.splitlines() if l.startswith("mus':")][0].split()[1])
    assert 1.0 <= mua <= 3.0 and 20.0 <= mus <= 40.0, r.stdout


@pytest.mark.gpu
def test_lookup_program_reference_example(programs, tmp_path):
    """The reference's example table (--example: 13 x 11 grid, 1e5 packets,
    10 runs, separate spheres) writes both CSVs with finite averages and
    standard errors, R_d falling with mu_a along every mu_s' column."""
    lookup, _ = programs
    r = _run([lookup, "--GPU", "0", "--example", "--go", "--seed", "5"], cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    Rm, Rse = _read_like_lookup_py(tmp_path / "Diffuse_Reflectance.csv", 13)
    Tm, Tse = _read_like_lookup_py(tmp_path / "Diffuse_Transmittance.csv", 13)
    assert Rm.shape == (13, 11) and Tm.shape == (13, 11)
    assert np.all(np.isfinite(Rm)) and np.all(np.isfinite(Tm))
    assert np.all(Rse > 0) and np.all(Rse < 0.01) and np.all(Tse < 0.01)
    assert np.all(np.diff(Rm, axis=0) < 0)
