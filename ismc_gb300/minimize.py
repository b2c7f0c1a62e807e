"""The minimisation driver's outer loops (Minimization/minimization.py:159-283)
on the batched solver.

The reference draws O samples of the refractive index, the sphere parameters
and the measurements from normal distributions, and for each sample runs
`runs` minimisations from the same initial guess, keeping only answers inside
the accepted box (retrying otherwise).  It then reports the mean and standard
deviation over samples of the per-sample mean.  Here every (sample, repeat)
minimisation is one entry of a single ismc_solve_batch call, so all of them
advance together and each round of objective evaluations is one GPU launch.
"""
import numpy as np

from .api import Engine, default_engine, make_solve


def minimize_distribution(layers, layer, samples, measurements, N, runs=1, x0=(5.0, 45.0),
                          lo=(1.0, 20.0), hi=(3.0, 40.0), separate=False, seed=0,
                          log_coords=True, max_evals=400, max_restarts=8, engine: Engine = None):
    """samples: list of (n, Spheres) (lookup.sample_distributions);
    measurements: array [O x 4] of (R_d, R_s, T_d, T_u), NaN = not measured.
    The index of `layer` in `layers` gets n and the unknown (mu_a, mu_s').
    Returns dict with per-sample means (mu_a, mu_s'), the final
    mean/std over samples (minimization.py:276-283) and per-solve outputs."""
    eng = engine or default_engine()
    meas = np.asarray(measurements, dtype=float)
    reqs, key = [], []
    for r, (n_r, sph) in enumerate(samples):
        ls = list(layers)
        L = ls[layer]
        ls[layer] = type(L)(n_r, L.mua, L.mus, L.g, L.d)
        m = [None if np.isnan(v) else float(v) for v in meas[r]]
        for i in range(runs):
            reqs.append(make_solve(ls, layer, sph, N, m, x0=x0, lo=lo, hi=hi,
                                   seed=seed + 1000 * r + i, separate=separate,
                                   log_coords=log_coords, max_evals=max_evals,
                                   max_restarts=max_restarts))
            key.append(r)
    out = eng.solve_batch(reqs)
    O = len(samples)
    mua = np.full(O, np.nan)
    mus = np.full(O, np.nan)
    for r in range(O):
        xs = [o.x for o, k in zip(out, key) if k == r and o.status == 0]
        if xs:
            mua[r] = np.mean([x[0] for x in xs])
            mus[r] = np.mean([x[1] for x in xs])
    return {"mu_a_per_sample": mua, "mu_s_per_sample": mus,
            "mu_a": float(np.nanmean(mua)), "mu_a_unc": float(np.nanstd(mua)),
            "mu_s": float(np.nanmean(mus)), "mu_s_unc": float(np.nanstd(mus)),
            "solves": out}
