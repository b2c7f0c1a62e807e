"""Batched lookup-table generation: the caller of the forward model in
Lookup/lookup.py:228-259 (sample_space) and CUDA/ISMLMC-lookup.cu:153-421
(singleLayerSampleSpace), done as ONE persistent launch over every grid point,
repeat and sphere configuration instead of one simulation at a time.

``sample_space`` keeps the reference's semantics: for each (mu_a_i, mu_s'_j)
and each of `runs` repeats it simulates N packets, either once with both
spheres (separate=False) or twice -- R sphere only and T sphere only
(separate=True, lookup.py:248-251) -- and returns the mean and the standard
deviation over repeats of R_d and T_d, arrays of shape (len(mu_a), len(mu_s')),
as lookup.py:254-257 does (np.std, ddof=0).
"""
import ctypes as C

import numpy as np

from . import _abi
from .api import (IsmcError, Layer, Spheres, default_engine, load_library, make_instance,
                  tallies_mean_se)


def _slab(n, mua, mus, g, t, slides):
    tissue = Layer(n, mua, mus, g, t)
    if slides is None:
        return [tissue]
    return [slides[0], tissue, slides[1]]


_KIND_R, _KIND_T, _KIND_RT = 0, 1, 2


def _grid_fill(v, mu_a, mu_s_reduced, g, t, n, spheres, N, runs, separate, seed, stream0,
               slides, mode):
    """Fill v (a numpy view of consecutive ismc_instance entries) with one
    sample_space grid, in (mu_a, mu_s', repeat, sphere) order with Philox
    streams stream0, stream0+1, ..., so a grid run alone or inside a larger
    batch gives the same tallies.  Returns the (i, j, repeat, kind) index."""
    mu_a = np.asarray(mu_a, dtype=float)
    musr = np.asarray(mu_s_reduced, dtype=float)
    mus = musr / (1 - g) if g != 1 else musr          # lookup.py:236
    thr = 1e-3 if slides is None else 1e-4
    if separate:
        kinds = ((_KIND_R, Spheres(**{**spheres.__dict__, "T": False})),
                 (_KIND_T, Spheres(**{**spheres.__dict__, "R": False})))
    else:
        kinds = ((_KIND_RT, spheres),)
    K, na, ns = len(kinds), len(mu_a), len(mus)
    rows = np.arange(na * ns * runs * K)
    i = rows // (ns * runs * K)
    j = (rows // (runs * K)) % ns
    r = (rows // K) % runs
    k = rows % K
    li = 0 if slides is None else 1                   # the tissue layer
    for kk, (code, sp) in enumerate(kinds):
        tmpl = (_abi.Instance * 1)(make_instance(_slab(n, float(mu_a[0]), float(mus[0]), g, t, slides),
                                                 sp, N, seed=seed, stream=0, mode=mode,
                                                 roulette_threshold=thr))
        v[k == kk] = np.ctypeslib.as_array(tmpl)[0]
    st = v["stack"]
    st["mua"][:, li] = mu_a[i]
    st["mus"][:, li] = mus[j]
    st["mut"][:, li] = mu_a[i] + mus[j]
    v["stream"] = (rows.astype(np.uint64) + np.uint64(stream0)) & np.uint64(0xFFFFFFFF)
    which = np.array([c for c, _ in kinds])[k]
    return {"i": i, "j": j, "r": r, "which": which}


def _grid_instances(mu_a, mu_s_reduced, g, t, n, spheres, N, runs, separate, seed, stream0,
                    slides, mode):
    """The instances of one sample_space grid (a ctypes array) and their index."""
    count = len(mu_a) * len(mu_s_reduced) * runs * (2 if separate else 1)
    arr = (_abi.Instance * count)()
    index = _grid_fill(np.ctypeslib.as_array(arr), mu_a, mu_s_reduced, g, t, n, spheres, N, runs,
                       separate, seed, stream0, slides, mode)
    return arr, index


def _grid_tables(res, index, shape):
    """R_d and T_d of every (mu_a, mu_s', repeat) from the batch's results
    (a ctypes tally array or a list of Result)."""
    if isinstance(res, C.Array):
        mean = tallies_mean_se(res)[0]
    else:
        mean = np.array([x.mean for x in res], dtype=float)
    return _grid_tables_from_mean(mean, index, shape)


def _grid_tables_from_mean(mean, index, shape):
    Rd = np.zeros(shape)
    Td = np.zeros(shape)
    i, j, r, w = index["i"], index["j"], index["r"], index["which"]
    m = w != _KIND_T
    Rd[i[m], j[m], r[m]] = mean[m, 1]
    m = w != _KIND_R
    Td[i[m], j[m], r[m]] = mean[m, 3]
    return Rd, Td


def sample_space(mu_a, mu_s_reduced, g, t, n, spheres: Spheres, N, runs=1, separate=True,
                 seed=0, slides=None, mode="compat", engine=None, tune=None):
    """R_d, R_d_std, T_d, T_d_std over the (mu_a x mu_s') grid in one launch.

    slides: None for the bare slab (ISMC.py single-slab walk, roulette 1e-3,
    as lookup.py's pythonISMC), or a (top, bottom) pair of Layer slides
    (multilayer walk, roulette 1e-4, as ISMLMC.py)."""
    eng = engine or default_engine()
    insts, index = _grid_instances(mu_a, mu_s_reduced, g, t, n, spheres, N, runs, separate, seed,
                                   0, slides, mode)
    Rd, Td = _grid_tables(eng.run_batch_raw(insts, tune), index,
                          (len(mu_a), len(mu_s_reduced), runs))
    return Rd.mean(-1), Rd.std(-1), Td.mean(-1), Td.std(-1)


SPHERE_KEYS = ("R_pw", "R_fs", "R_fp", "R_fd", "R_angle", "T_pw", "T_fs", "T_fp", "T_fd", "T_angle")


def sample_distributions(n, n_unc, spheres: Spheres, spheres_unc: dict, O, seed=0):
    """O draws of the refractive index and of the sphere parameters from normal
    distributions (lookup.py:133-143, minimization.py:132-152); spheres_unc
    maps parameter names (SPHERE_KEYS) to standard deviations.  Total port
    fractions follow their parts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_dist = rng.normal(n, n_unc, O)
    draws = {k: rng.normal(getattr(spheres, k), spheres_unc.get(k, 0.0), O) for k in SPHERE_KEYS}
    out = []
    for r in range(O):
        d = {**spheres.__dict__, **{k: float(v[r]) for k, v in draws.items()}}
        d["R_f"] = d["R_fs"] + d["R_fp"] + d["R_fd"]
        d["T_f"] = d["T_fs"] + d["T_fp"] + d["T_fd"]
        out.append((float(n_dist[r]), Spheres(**d)))
    return out


def run_uncertainty(mu_a, mu_s_reduced, g, t, samples, N, runs=1, separate=True, seed=0,
                    slides=None, mode="compat", engine=None, tune=None):
    """lookup.py:263-293 (runPYTHON) as ONE launch: for every drawn (n, spheres)
    in `samples` the whole grid with `runs` repeats.  Returns the mean over
    samples of R_d and T_d and their spread: sqrt(sum of per-sample repeat
    variances) when runs > 1, else the standard deviation over samples."""
    eng = engine or default_engine()
    per = len(mu_a) * len(mu_s_reduced) * runs * (2 if separate else 1)
    arr = (_abi.Instance * (per * len(samples)))()
    v = np.ctypeslib.as_array(arr)
    indices = [_grid_fill(v[r * per:(r + 1) * per], mu_a, mu_s_reduced, g, t, n_r, sph_r, N, runs,
                          separate, seed, r * per, slides, mode)
               for r, (n_r, sph_r) in enumerate(samples)]
    res = eng.run_batch_raw(arr, tune)
    O = len(samples)
    shape = (len(mu_a), len(mu_s_reduced), runs)
    Rd, Td = np.zeros((O,) + shape[:2]), np.zeros((O,) + shape[:2])
    Rv, Tv = np.zeros(shape[:2]), np.zeros(shape[:2])
    mean = tallies_mean_se(res)[0]
    for r, index in enumerate(indices):
        R3, T3 = _grid_tables_from_mean(mean[r * per:(r + 1) * per], index, shape)
        Rd[r], Td[r] = R3.mean(-1), T3.mean(-1)
        Rv += R3.std(-1) ** 2
        Tv += T3.std(-1) ** 2
    if runs > 1:
        Rs, Ts = np.sqrt(Rv), np.sqrt(Tv)
    else:
        Rs, Ts = Rd.std(0), Td.std(0)
    return Rd.mean(0), Rs, Td.mean(0), Ts


# ----------------------------------------------------------------------------
# lookup-table inversion on the GPU (Lookup/lookup.py:301-489)
# ----------------------------------------------------------------------------
def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def _rc(rc):
    if rc:
        buf = C.create_string_buffer(512)
        load_library().ismc_last_error(None, buf, 512)
        raise IsmcError(rc, buf.value.decode(errors="replace"))


def table_grid(N):
    """The table axis in percent: np.linspace(0, 100, N) (lookup.py:347-348)."""
    return np.linspace(0, 100, N)


def _i32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def interp_table(R, T, values, N=1000, tri=None, method="cubic"):
    """Scattered samples (R, T in percent, value) -> N x N table indexed [R_i][T_j],
    NaN outside the samples' convex hull, as scipy.interpolate.griddata makes it
    (lookup.py:339-342).  method "cubic" (Clough-Tocher, griddata's cubic) or
    "linear" (barycentric).  tri: a scipy.spatial.Delaunay of the points (built
    here when None; for "linear" an [ntri x 3] simplex array also works)."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    v = np.ascontiguousarray(values, dtype=np.float64)
    if tri is None:
        from scipy.spatial import Delaunay
        tri = Delaunay(np.stack([R, T], 1))
    out = np.empty((N, N))
    optr = out.ctypes.data_as(C.POINTER(C.c_double))
    lib = load_library()
    if method == "linear":
        simp = np.ascontiguousarray(getattr(tri, "simplices", tri), dtype=np.int32)
        _rc(lib.ismc_table_interp(_dp(R), _dp(T), _dp(v), len(R), _i32p(simp), len(simp), N, optr))
    elif method == "cubic":
        simp = np.ascontiguousarray(tri.simplices, dtype=np.int32)
        nbr = np.ascontiguousarray(tri.neighbors, dtype=np.int32)
        ptr, adj = (np.ascontiguousarray(a, dtype=np.int32) for a in tri.vertex_neighbor_vertices)
        _rc(lib.ismc_table_interp_cubic(_dp(R), _dp(T), _dp(v), len(R), _i32p(simp), _i32p(nbr),
                                        len(simp), _i32p(ptr), _i32p(adj), N, optr))
    else:
        raise ValueError(f"method must be 'cubic' or 'linear', not {method!r}")
    return out


def uncertainty_map(mua_table, mus_table, rstd_table, tstd_table, M=100, seed=0):
    """Per-cell percent uncertainty of the mu_a and mu_s' tables from M Gaussian
    draws of (R, T) (lookup.py:349-376); tables [R_i][T_j]."""
    N = mua_table.shape[0]
    a, b = np.empty((N, N)), np.empty((N, N))
    _rc(load_library().ismc_table_uncertainty(_dp(mua_table), _dp(mus_table), _dp(rstd_table),
                                              _dp(tstd_table), N, int(M), int(seed),
                                              a.ctypes.data_as(C.POINTER(C.c_double)),
                                              b.ctypes.data_as(C.POINTER(C.c_double))))
    return a, b


def lookup(table_t, R, T):
    """Nearest-cell values of the transposed table table_t[T_j][R_i] for arrays of
    measurements R, T in percent (lookup.py:467-489, vectorised)."""
    N = table_t.shape[0]
    R = np.atleast_1d(np.asarray(R, dtype=np.float64))
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    out = np.empty(len(R))
    _rc(load_library().ismc_table_lookup(_dp(table_t), N, _dp(R), _dp(T), len(R),
                                         out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def make_lookup(refl, trans, refl_std, trans_std, mu_a, mu_s_reduced, N=1000, uncertainty=True,
                M=100, seed=0, skip_first=True, method="cubic"):
    """lookup.py:301-465 `makelookup` on the GPU: the (R, T) -> mu_a and mu_s'
    tables, the interpolated R/T standard deviations and the uncertainty maps.
    As the reference does, the first row and column of the grid are skipped
    (lookup.py:307-310; skip_first), the samples are ordered by R then T
    (lookup.py:320-323) and interpolated with griddata's method (cubic by
    default).  Returns the transposed tables as the reference does: (mua_t,
    mua_unc_t, mus_t, mus_unc_t, Rvals, Tvals)."""
    refl, trans = np.asarray(refl, float), np.asarray(trans, float)
    s = 1 if skip_first else 0
    I, J = np.meshgrid(np.arange(s, refl.shape[0]), np.arange(s, refl.shape[1]), indexing="ij")
    R = 100 * refl[I, J].ravel()
    T = 100 * trans[I, J].ravel()
    order = np.lexsort((T, R))          # stable sort by R, then T
    R, T, I, J = R[order], T[order], I.ravel()[order], J.ravel()[order]
    from scipy.spatial import Delaunay
    tri = Delaunay(np.stack([R, T], 1))
    mua_t = interp_table(R, T, np.asarray(mu_a, float)[I], N, tri, method)
    mus_t = interp_table(R, T, np.asarray(mu_s_reduced, float)[J], N, tri, method)
    if uncertainty:
        rs = interp_table(R, T, 100 * np.asarray(refl_std, float)[I, J], N, tri, method)
        ts = interp_table(R, T, 100 * np.asarray(trans_std, float)[I, J], N, tri, method)
        ua, us = uncertainty_map(mua_t, mus_t, rs, ts, M, seed)
    else:
        ua = us = np.full((N, N), np.nan)
    grid = table_grid(N)
    return mua_t.T, ua.T, mus_t.T, us.T, grid, grid
