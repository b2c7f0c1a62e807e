"""Lookup-table inversion on the GPU (Lookup/lookup.py:301-489): cubic
(Clough-Tocher) and linear interpolation against scipy's griddata on the same
triangulation, the cubic one also against the FP64 restatement, the Monte
Carlo uncertainty map against the FP64 numpy restatement with the same normal
draws (oracle/table64.py), and the nearest-cell lookup."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scattered(n=40, seed=0):
    rng = np.random.default_rng(seed)
    a, b = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    R = 5 + 50 * a + 3 * np.sin(3 * b) + rng.normal(0, 0.2, a.shape)
    T = 2 + 25 * b * (1 - 0.5 * a) + rng.normal(0, 0.2, a.shape)
    v = np.exp(0.5 * a) * (1 + b ** 2)
    return R.ravel(), T.ravel(), v.ravel()


def test_interp_matches_scipy_linear():
    from scipy.interpolate import griddata
    from scipy.spatial import Delaunay
    from ismc_gb300.lookup import interp_table, table_grid
    R, T, v = _scattered()
    N = 301
    tri = Delaunay(np.stack([R, T], 1))
    got = interp_table(R, T, v, N, tri.simplices, method="linear")
    g = table_grid(N)
    gx, gy = np.meshgrid(g, g, indexing="ij")
    ref = griddata(np.stack([R, T], 1), v, (gx, gy), method="linear")
    both = np.isfinite(got) & np.isfinite(ref)
    assert np.max(np.abs(got[both] - ref[both])) < 1e-9
    # NaN masks differ at most on cells lying on the hull boundary
    assert np.mean(np.isfinite(got) != np.isfinite(ref)) < 2e-3
    assert both.sum() > 0.05 * N * N          # the samples' hull covers ~10 % of the table


@pytest.mark.parametrize("seed", [0, 1])
def test_interp_cubic_matches_scipy_and_oracle(seed):
    """griddata(method="cubic") is what lookup.py interpolates with: the GPU
    Clough-Tocher table agrees with it, cell for cell, to rounding."""
    from scipy.interpolate import griddata
    from oracle import table64
    from ismc_gb300.lookup import interp_table, table_grid
    R, T, v = _scattered(n=30, seed=seed)
    order = np.lexsort((T, R))
    R, T, v = R[order], T[order], v[order]
    N = 201
    got = interp_table(R, T, v, N, method="cubic")
    g = table_grid(N)
    gx, gy = np.meshgrid(g, g, indexing="ij")
    ref = griddata(np.stack([R, T], 1), v, (gx, gy), method="cubic")
    both = np.isfinite(got) & np.isfinite(ref)
    scale = np.max(np.abs(ref[both]))
    assert np.max(np.abs(got[both] - ref[both])) < 1e-9 * scale
    assert np.mean(np.isfinite(got) != np.isfinite(ref)) < 2e-3
    assert both.sum() > 0.05 * N * N
    if seed == 0:                      # the FP64 restatement on a coarser table
        Nc = 41
        oc = table64.cubic_table(R, T, v, Nc)
        gc = interp_table(R, T, v, Nc, method="cubic")
        bc = np.isfinite(oc) & np.isfinite(gc)
        assert bc.sum() > 0 and np.max(np.abs(oc[bc] - gc[bc])) < 1e-9 * scale


def test_interp_cubic_reproduces_linear_data():
    """A linear function has zero curvature: the gradient estimate converges to
    the exact gradient and the cubic table equals the function inside the hull,
    to the estimate's convergence tolerance (1e-6 relative change per sweep)."""
    from ismc_gb300.lookup import interp_table, table_grid
    R, T, _ = _scattered(n=20, seed=3)
    v = 0.3 + 0.02 * R - 0.05 * T
    N = 101
    got = interp_table(R, T, v, N, method="cubic")
    g = table_grid(N)
    gx, gy = np.meshgrid(g, g, indexing="ij")
    f = np.isfinite(got)
    assert f.sum() > 0
    assert np.max(np.abs(got[f] - (0.3 + 0.02 * gx[f] - 0.05 * gy[f]))) < 1e-6


def test_uncertainty_map_matches_oracle():
    from oracle import table64
    from ismc_gb300.lookup import uncertainty_map
    N, M = 24, 64
    rng = np.random.default_rng(1)
    g = np.linspace(0, 1, N)
    A, B = np.meshgrid(g, g, indexing="ij")
    mua = 0.1 + A + 0.5 * B
    mus = 10 + 20 * B * (1 + A)
    rs = np.abs(rng.normal(3, 1, (N, N)))
    ts = np.abs(rng.normal(2, 1, (N, N)))
    rs[3, 5] = np.nan
    ts[7, 2] = -1.0
    mua[10, 10] = np.nan              # NaN table cells poison the draws that land there
    ua, us = uncertainty_map(mua, mus, rs, ts, M=M, seed=12345)
    oa, os_ = table64.uncertainty_map(mua, mus, rs, ts, M, 12345)
    for got, ref in ((ua, oa), (us, os_)):
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        f = np.isfinite(ref)
        rel = np.abs(got[f] - ref[f]) / np.maximum(np.abs(ref[f]), 1e-300)
        assert np.mean(rel < 1e-9) > 0.995, np.sort(rel)[-5:]


def test_lookup_nearest_cell():
    from oracle import table64
    from ismc_gb300.lookup import lookup, table_grid
    N = 101
    rng = np.random.default_rng(2)
    table_t = rng.random((N, N))
    R = rng.uniform(-5, 105, 500)
    T = rng.uniform(-5, 105, 500)
    got = lookup(table_t, R, T)
    g = table_grid(N)
    ref = [table_t[table64.find_nearest(g, t)][table64.find_nearest(g, r)] for r, t in zip(R, T)]
    assert np.array_equal(got, np.array(ref))


def test_uncertainty_runs_in_one_launch_equal_the_loop(engine):
    """lookup.py:263-293 folded into one batch gives exactly the per-sample
    loop's numbers (streams are keyed by position in the grid)."""
    from ismc_gb300.lookup import _grid_instances, _grid_tables, run_uncertainty, sample_distributions
    from ismc_gb300.workloads import bench_spheres
    mu_a, mus_r = [0.5, 1.0, 3.0], [10.0, 20.0]
    samples = sample_distributions(1.4, 0.02, bench_spheres(), {"R_pw": 0.005, "T_pw": 0.005,
                                                                 "R_fs": 0.001}, 5, seed=9)
    for runs in (1, 3):
        Rd, Rs, Td, Ts = run_uncertainty(mu_a, mus_r, 0.9, 0.1, samples, 20_000, runs=runs, seed=4,
                                         engine=engine)
        per = len(mu_a) * len(mus_r) * runs * 2
        R_all, T_all, Rv, Tv = [], [], 0, 0
        for r, (n_r, sp) in enumerate(samples):
            insts, index = _grid_instances(mu_a, mus_r, 0.9, 0.1, n_r, sp, 20_000, runs, True, 4,
                                           r * per, None, "compat")
            R3, T3 = _grid_tables(engine.run_batch(insts), index, (3, 2, runs))
            R_all.append(R3.mean(-1)); T_all.append(T3.mean(-1))
            Rv = Rv + R3.std(-1) ** 2; Tv = Tv + T3.std(-1) ** 2
        assert np.array_equal(Rd, np.mean(R_all, 0)) and np.array_equal(Td, np.mean(T_all, 0))
        if runs > 1:
            assert np.array_equal(Rs, np.sqrt(Rv)) and np.array_equal(Ts, np.sqrt(Tv))
        else:
            assert np.array_equal(Rs, np.std(R_all, 0))


def test_make_lookup_inverts_the_generating_grid(engine):
    """End to end: batched lookup generation on a small grid, then the GPU
    tables map each grid point's (R, T) back near its own (mu_a, mu_s')."""
    from ismc_gb300.lookup import lookup, make_lookup, sample_space
    from ismc_gb300.workloads import bench_spheres
    from ismc_gb300 import Layer
    mu_a = 0.5 * 1.2 ** np.arange(10)
    mus_r = 10 * 1.2 ** np.arange(9)
    sl = (Layer.slide(1.5, 0.1), Layer.slide(1.5, 0.1))
    Rd, Rs, Td, Ts = sample_space(mu_a, mus_r, 0.9, 0.135, 1.4, bench_spheres(), 100_000, runs=4,
                                  separate=True, seed=3, slides=sl, engine=engine)
    mua_t, ua, mus_t, us, Rv, Tv = make_lookup(Rd, Td, Rs, Ts, mu_a, mus_r, N=400, M=50, seed=1)
    I, J = np.meshgrid(np.arange(2, 9), np.arange(2, 8), indexing="ij")     # interior points
    ga = lookup(mua_t, 100 * Rd[I, J].ravel(), 100 * Td[I, J].ravel())
    gs = lookup(mus_t, 100 * Rd[I, J].ravel(), 100 * Td[I, J].ravel())
    assert np.median(np.abs(ga / mu_a[I].ravel() - 1)) < 0.05
    assert np.median(np.abs(gs / mus_r[J].ravel() - 1)) < 0.05
    assert np.isfinite(ua).mean() > 0.01 and np.nanmedian(ua) > 0
