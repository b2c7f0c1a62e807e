"""Shared argument handling of the drop-in modules."""
import itertools
import threading

from ismc_gb300 import api

_counter = itertools.count()
_lock = threading.Lock()
_base_seed = [0x15C0FFEE]


def seed(s):
    """Reset the call-sequence seed (the reference uses the global `random`
    state, ISMC.py:17; here call k of a process draws Philox stream k of the
    seed, so a seeded process is reproducible)."""
    global _counter
    with _lock:
        _base_seed[0] = int(s)
        _counter = itertools.count()


def next_stream():
    with _lock:
        return _base_seed[0], next(_counter)


def spheres_from_args(R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle, specular_included,
                      T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle):
    return api.Spheres(R=bool(R), R_pw=float(R_pw), R_fs=float(R_fs), R_fp=float(R_fp),
                       R_fd=float(R_fd), R_f=float(R_f), R_angle=float(R_angle),
                       specular_included=bool(specular_included), T=bool(T), T_pw=float(T_pw),
                       T_fs=float(T_fs), T_fp=float(T_fp), T_fd=float(T_fd), T_f=float(T_f),
                       T_angle=float(T_angle))


def run(layers, spheres, N, roulette_threshold, seed=None, mode="compat", engine=None):
    N = int(N)
    if N <= 0:
        raise ZeroDivisionError("N must be positive (the reference divides by N)")
    base, stream = next_stream()
    if seed is not None:
        base, stream = int(seed), 0
    inst = api.make_instance(layers, spheres, N, seed=base, stream=stream, mode=mode,
                             roulette_threshold=roulette_threshold, roulette_m=10.0)
    eng = engine or api.default_engine()
    res = eng.run_batch([inst])[0]
    return res
