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


def uncertainty_map(mua, mus, rstd, tstd, M, seed, cells=None):
    """mua/mus/rstd/tstd: [N x N] tables indexed [R_i][T_j] (percent grid).
    cells: optional (i, j) pairs to evaluate (the others stay NaN)."""
    N = mua.shape[0]
    grid = np.linspace(0, 100, N)
    k0, k1 = seed & MASK, (seed >> 32) & MASK
    ua = np.full((N, N), np.nan)
    us = np.full((N, N), np.nan)
    todo = cells if cells is not None else ((i, j) for i in range(N) for j in range(N))
    for i, j in todo:
        if True:
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


# ---------------------------------------------------------------------------
# Cubic (Clough-Tocher) interpolation of scattered samples, the method of
# scipy.interpolate.griddata(method="cubic") that lookup.py:339-342 uses.
# Restated from the published construction:
#   * vertex gradients minimise the summed squared second derivative of the
#     cubic Hermite interpolant along every triangulation edge (Nielson 1983;
#     Renka & Cline 1984), solved per vertex by Gauss-Seidel sweeps in vertex
#     order until the largest change, relative to max(1, |gradient|), is
#     below tol (at most maxiter sweeps);
#   * each triangle is split at its centroid into three cubic Bezier patches
#     (Clough-Tocher; Farin 1986): vertex values and gradients fix the
#     boundary control points, C1 across the inner edges fixes the rest once
#     the cross-boundary derivative of every outer edge is chosen; it is
#     chosen linear along the edge, taken in the direction from the
#     neighbouring triangle's centroid to this triangle's centroid (from the
#     edge midpoint to the centroid on the hull).
# ---------------------------------------------------------------------------
def ct_gradients(x, y, indptr, indices, maxiter=400, tol=1e-6):
    """Vertex gradients [n x 2] from points x [n x 2], values y [n] and the
    vertex adjacency in CSR form (scipy's vertex_neighbor_vertices)."""
    n = len(x)
    g = np.zeros((n, 2))
    for _ in range(maxiter):
        err = 0.0
        for i in range(n):
            j = indices[indptr[i]:indptr[i + 1]]
            e = x[j] - x[i]
            L3 = np.sqrt((e * e).sum(1)) ** 3
            q0 = (4 * e[:, 0] * e[:, 0] / L3).sum()
            q1 = (4 * e[:, 0] * e[:, 1] / L3).sum()
            q2 = (4 * e[:, 1] * e[:, 1] / L3).sum()
            w = (6 * (y[i] - y[j]) + 2 * (e * g[j]).sum(1)) / L3
            s0, s1 = (w * e[:, 0]).sum(), (w * e[:, 1]).sum()
            det = q0 * q2 - q1 * q1
            r0 = (q2 * s0 - q1 * s1) / det
            r1 = (-q1 * s0 + q0 * s1) / det
            change = max(abs(g[i, 0] + r0), abs(g[i, 1] + r1)) / max(1.0, abs(r0), abs(r1))
            g[i] = (-r0, -r1)
            err = max(err, change)
        if err < tol:
            break
    return g


def _ct_value(V, f, G, Vn, b):
    """Clough-Tocher value on triangle V [3 x 2] with values f, gradients G
    [3 x 2], neighbour centroids Vn [3 x 2] (row k: across the edge opposite
    vertex k; NaN on the hull) at barycentric coordinates b."""
    V0 = V.mean(0)
    c = {}
    # vertex and edge control points of the macro triangle (i j k: vertex weights)
    for a in range(3):
        c[a, a] = f[a]
    for a in range(3):
        for bb in range(3):
            if a != bb:
                c[a, bb] = f[a] + G[a].dot(V[bb] - V[a]) / 3      # next to vertex a toward bb
    inner = [(c[a, a] + c[a, (a + 1) % 3] + c[a, (a + 2) % 3]) / 3 for a in range(3)]
    cross = {}
    for a in range(3):
        bb = (a + 1) % 3
        k = 3 - a - bb
        VA, VB = V[a], V[bb]
        if np.isnan(Vn[k, 0]):
            al = be = -0.5
        else:
            d = V0 - Vn[k]
            A = np.array([[VA[0] - V0[0], VB[0] - V0[0]], [VA[1] - V0[1], VB[1] - V0[1]]])
            aa, b2 = np.linalg.solve(A, d)
            cc = -(aa + b2)
            al, be = aa / cc, b2 / cc
        q0 = al * c[a, a] + be * c[a, bb] + inner[a]
        q2 = al * c[bb, a] + be * c[bb, bb] + inner[bb]
        cross[a] = (q0 + q2) / 2 - al * c[a, bb] - be * c[bb, a]      # edge a -> a+1
    near = [(inner[a] + cross[a] + cross[(a + 2) % 3]) / 3 for a in range(3)]
    center = sum(near) / 3
    m = int(np.argmin(b))
    a, bb = (m + 1) % 3, (m + 2) % 3          # subtriangle (a, bb, centroid)
    u, v, w0 = b[a] - b[m], b[bb] - b[m], 3 * b[m]
    # Bernstein form on (a, bb, centroid); edge a->bb is cross[a] when bb == a+1
    cr = cross[a]
    pts = {(3, 0, 0): c[a, a], (2, 1, 0): c[a, bb], (1, 2, 0): c[bb, a], (0, 3, 0): c[bb, bb],
           (2, 0, 1): inner[a], (1, 1, 1): cr, (0, 2, 1): inner[bb],
           (1, 0, 2): near[a], (0, 1, 2): near[bb], (0, 0, 3): center}
    coef = {(3, 0, 0): 1, (0, 3, 0): 1, (0, 0, 3): 1, (1, 1, 1): 6}
    val = 0.0
    for (i, j, l), cp in pts.items():
        val += coef.get((i, j, l), 3) * u ** i * v ** j * w0 ** l * cp
    return val


def cubic_table(R, T, val, N):
    """N x N table over [0,100]^2 (indexed [R_i][T_j]) of the Clough-Tocher
    interpolant of the samples, NaN outside their convex hull."""
    from scipy.spatial import Delaunay
    P = np.stack([R, T], 1).astype(np.float64)
    tri = Delaunay(P)
    indptr, indices = tri.vertex_neighbor_vertices
    y = np.asarray(val, np.float64)
    G = ct_gradients(P, y, indptr, indices)
    cen = P[tri.simplices].mean(1)
    grid = np.linspace(0, 100, N)
    X, Y = np.meshgrid(grid, grid, indexing="ij")
    Q = np.stack([X.ravel(), Y.ravel()], 1)
    s = tri.find_simplex(Q)
    out = np.full(len(Q), np.nan)
    for k in np.nonzero(s >= 0)[0]:
        t = s[k]
        iv = tri.simplices[t]
        Tm = tri.transform[t]
        b01 = Tm[:2].dot(Q[k] - Tm[2])
        b = np.array([b01[0], b01[1], 1 - b01.sum()])
        nb = tri.neighbors[t]
        Vn = np.where((nb >= 0)[:, None], cen[np.maximum(nb, 0)], np.nan)
        out[k] = _ct_value(P[iv], y[iv], G[iv], Vn, b)
    return out.reshape(N, N)
