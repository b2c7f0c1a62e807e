"""Drop-in for the reference's ISMLMC.py (layer stack, ISMLMC.py:101-347).

    ISMLMC(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, ..., T_angle) -> (A, R_d, R_s, T_d, T_u)

n, g, t, mu_a, mu_s, mu_t are per-layer lists, top first; a layer with
mu_s == 0 is a slide (ISMLMC.py:81).  Roulette threshold 1e-4, m = 10
(MLMC.py:86-87).  Runs on the GPU through libismc.so.
"""
from ismc_gb300 import api
from ismc_gb300.dropin import _common
from ismc_gb300.dropin._common import seed  # noqa: F401


def _layers(n, g, t, mu_a, mu_s, mu_t):
    k = len(n)
    if not all(len(x) == k for x in (g, t, mu_a, mu_s, mu_t)):
        raise ValueError("n, g, t, mu_a, mu_s, mu_t must have the same length")
    return [api.Layer(float(n[i]), float(mu_a[i]), float(mu_s[i]), float(g[i]), float(t[i]),
                      float(mu_t[i])) for i in range(k)]


def ISMLMC_ex(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
              specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle, seed=None,
              mode="compat"):
    """As ISMLMC() but returns (means[5], standard_errors[5], status)."""
    sp = _common.spheres_from_args(R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle, specular_included,
                                   T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle)
    r = _common.run(_layers(n, g, t, mu_a, mu_s, mu_t), sp, N, 1e-4, seed=seed, mode=mode)
    return tuple(r.mean), tuple(r.se), r.status


def ISMLMC(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f, R_angle,
           specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle):
    means, _, _ = ISMLMC_ex(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, R_fs, R_fp, R_fd, R_f,
                            R_angle, specular_included, T, T_pw, T_fs, T_fp, T_fd, T_f, T_angle)
    return means
