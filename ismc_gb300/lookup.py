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
import numpy as np

from .api import Layer, Spheres, default_engine, make_instance


def _slab(n, mua, mus, g, t, slides):
    tissue = Layer(n, mua, mus, g, t)
    if slides is None:
        return [tissue]
    return [slides[0], tissue, slides[1]]


def sample_space(mu_a, mu_s_reduced, g, t, n, spheres: Spheres, N, runs=1, separate=True,
                 seed=0, slides=None, mode="compat", engine=None, tune=None):
    """R_d, R_d_std, T_d, T_d_std over the (mu_a x mu_s') grid in one launch.

    slides: None for the bare slab (ISMC.py single-slab walk, roulette 1e-3,
    as lookup.py's pythonISMC), or a (top, bottom) pair of Layer slides
    (multilayer walk, roulette 1e-4, as ISMLMC.py)."""
    eng = engine or default_engine()
    mu_a = np.asarray(mu_a, dtype=float)
    musr = np.asarray(mu_s_reduced, dtype=float)
    mus = musr / (1 - g) if g != 1 else musr          # lookup.py:236
    thr = 1e-3 if slides is None else 1e-4
    sp_R = Spheres(**{**spheres.__dict__, "T": False})
    sp_T = Spheres(**{**spheres.__dict__, "R": False})
    insts, index = [], []
    stream = 0
    for i, a in enumerate(mu_a):
        for j, s in enumerate(mus):
            layers = _slab(n, float(a), float(s), g, t, slides)
            for r in range(runs):
                if separate:
                    for which, sp in (("R", sp_R), ("T", sp_T)):
                        insts.append(make_instance(layers, sp, N, seed=seed, stream=stream,
                                                   mode=mode, roulette_threshold=thr))
                        index.append((i, j, r, which))
                        stream += 1
                else:
                    insts.append(make_instance(layers, spheres, N, seed=seed, stream=stream,
                                               mode=mode, roulette_threshold=thr))
                    index.append((i, j, r, "RT"))
                    stream += 1
    res = eng.run_batch(insts, tune)
    Rd = np.zeros((len(mu_a), len(mus), runs))
    Td = np.zeros((len(mu_a), len(mus), runs))
    for (i, j, r, which), x in zip(index, res):
        if which in ("R", "RT"):
            Rd[i, j, r] = x.mean[1]
        if which in ("T", "RT"):
            Td[i, j, r] = x.mean[3]
    return Rd.mean(-1), Rd.std(-1), Td.mean(-1), Td.std(-1)
