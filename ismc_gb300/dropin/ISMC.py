"""Drop-in for the reference's ISMC.py (single slab, ISMC.py:164-406).

    ISMC(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
         specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle)
        -> (A, R_d, R_s, T_d, T_u)   as fractions of N

Same argument meaning (angles in radians, R/T bool or 0/1, mu_t as passed by
the caller), same return order.  The walk uses the single-slab driver's
roulette threshold 1e-3 with m = 10 (ISMC.py:136).  Runs on the GPU through
libismc.so; raises if the library or the GPU is missing.
"""
from ismc_gb300 import api
from ismc_gb300.dropin import _common
from ismc_gb300.dropin._common import seed  # noqa: F401


def _layers(n, g, t, mu_a, mu_s, mu_t):
    return [api.Layer(float(n), float(mu_a), float(mu_s), float(g), float(t), float(mu_t))]


def ISMC_ex(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
            specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle, seed=None,
            mode="compat"):
    """As ISMC() but returns (means[5], standard_errors[5], status)."""
    sp = _common.spheres_from_args(R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle, specular_included,
                                   T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle)
    r = _common.run(_layers(n, g, t, mu_a, mu_s, mu_t), sp, N, 1e-3, seed=seed, mode=mode)
    return tuple(r.mean), tuple(r.se), r.status


def ISMC(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
         specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle):
    means, _, _ = ISMC_ex(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
                          specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle)
    return means
