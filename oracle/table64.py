"""ORACLE (test infrastructure only): FP64 numpy restatement of the lookup
table's Monte Carlo uncertainty map (Lookup/lookup.py:349-376), drawing the
same Philox4x32-10 normals as the GPU kernel (Box-Muller), so the two can be
compared cell by cell.  Also the reference's nearest-index rule
(lookup.py:296-299, np.argmin of |grid - value|).
"""
import numpy as np

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint64 arrays holding 32-bit words."""
    c = [np.asarray(x, dtype=np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0), np.uint64(k1)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
            k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        c = [(p1 >> np.uint64(32)) ^ c[1] ^ k0, p1 & np.uint64(MASK),
             (p0 >> np.uint64(32)) ^ c[3] ^ k1, p0 & np.uint64(MASK)]
    return c


def normal2(a, b):
    u1 = (a.astype(np.float64) + 0.5) * 2.0 ** -32
    u2 = (b.astype(np.float64) + 0.5) * 2.0 ** -32
    r = np.sqrt(-2.0 * np.log(u1))
    return r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)


def find_nearest(grid, v):
    return int(np.abs(np.asarray(grid) - v).argmin())


def uncertainty_map(mua, mus, rstd, tstd, M, seed):
    """mua/mus/rstd/tstd: [N x N] tables indexed [R_i][T_j] (percent grid)."""
    N = mua.shape[0]
    grid = np.linspace(0, 100, N)
    k0, k1 = seed & MASK, (seed >> 32) & MASK
    ua = np.full((N, N), np.nan)
    us = np.full((N, N), np.nan)
    for i in range(N):
        for j in range(N):
            sR, sT = rstd[i, j], tstd[i, j]
            if np.isnan(sR) or np.isnan(sT) or sR < 0 or sT < 0:
                continue
            k = i * N + j
            d = np.arange(0, M, 2, dtype=np.uint64)
            w = philox4x32_10(d, np.full_like(d, k & MASK), np.full_like(d, k >> 32),
                              np.full_like(d, 0x7AB1E5), k0, k1)
            zr = np.stack(normal2(w[0], w[1]), 1).ravel()[:M]
            zt = np.stack(normal2(w[2], w[3]), 1).ravel()[:M]
            va = [mua[find_nearest(grid, grid[i] + sR * a), find_nearest(grid, grid[j] + sT * b)]
                  for a, b in zip(zr, zt)]
            vs = [mus[find_nearest(grid, grid[i] + sR * a), find_nearest(grid, grid[j] + sT * b)]
                  for a, b in zip(zr, zt)]
            ua[i, j] = 100 * np.std(va) / mua[i, j]
            us[i, j] = 100 * np.std(vs) / mus[i, j]
    return ua, us
