// ismc_table.cu -- lookup-table inversion on the GPU (the step after batched
// lookup generation in Lookup/lookup.py:301-489).
//
//  ismc_table_interp       scattered (R, T) -> value samples interpolated onto
//                          the uniform N x N table over [0,100]% x [0,100]%
//                          (lookup.py:307-345, scipy griddata).  Linear
//                          (barycentric) interpolation on a triangulation the
//                          caller supplies (Delaunay, e.g. scipy.spatial), NaN
//                          outside it.  Point location: a uniform bucket grid
//                          over the triangles' bounding boxes, built on the host.
//  ismc_table_interp_cubic the same table by Clough-Tocher cubic interpolation,
//                          the method of griddata(method="cubic") that lookup.py
//                          uses: vertex gradients from the global curvature-
//                          minimising estimate (host, Gauss-Seidel), then one
//                          thread per cell evaluates the cubic Bezier patch of
//                          the Clough-Tocher split of its triangle.
//  ismc_table_uncertainty  per table cell, M Gaussian draws of (R, T) around the
//                          cell with the interpolated standard deviations, the
//                          nearest-cell values of the mu_a and mu_s' tables, and
//                          100 * std / value (lookup.py:349-376), one thread per
//                          cell, Philox4x32-10 normals (Box-Muller).
//  ismc_table_lookup       nearest-cell lookup of many (R, T) (lookup.py:467-489).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "ismc_dev.h"
#include "ismc_math.cuh"

namespace {

// nearest index of x on the grid 0, h, 2h, ..., 100 (N points): the first
// minimiser of |grid - x|, as np.argmin picks it
__device__ __forceinline__ int nearest_idx(double x, int N) {
    const double h = 100.0 / (N - 1);
    double t = x / h;
    if (!(t > 0.0)) return 0;                       // also NaN -> 0 (argmin of NaNs is 0)
    if (t >= N - 1) return N - 1;
    const double f = floor(t);
    int i = (int)f;
    const double lo = fabs(x - i * h), hi = fabs(x - (i + 1) * h);
    return hi < lo ? i + 1 : i;
}

__global__ void interp_kernel(const double* __restrict__ px, const double* __restrict__ py,
                              const double* __restrict__ val, const int* __restrict__ tri,
                              const int* __restrict__ bstart, const int* __restrict__ blist,
                              int nb, int N, double* __restrict__ out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long long)N * N) return;
    const int i = (int)(k / N), j = (int)(k % N);
    const double h = 100.0 / (N - 1);
    const double x = i * h, y = j * h;        // R = x, T = y, as np.mgrid[0:100:Nj] spaces them
    int bx = (int)(x / 100.0 * nb), by = (int)(y / 100.0 * nb);
    bx = min(max(bx, 0), nb - 1);
    by = min(max(by, 0), nb - 1);
    const int b = by * nb + bx;
    double res = NAN;
    const double eps = 1e-12;
    for (int q = bstart[b]; q < bstart[b + 1]; ++q) {
        const int t = blist[q];
        const int a0 = tri[3 * t], a1 = tri[3 * t + 1], a2 = tri[3 * t + 2];
        const double x0 = px[a0], y0 = py[a0], x1 = px[a1], y1 = py[a1], x2 = px[a2], y2 = py[a2];
        const double det = (y1 - y2) * (x0 - x2) + (x2 - x1) * (y0 - y2);
        if (det == 0.0) continue;
        const double l0 = ((y1 - y2) * (x - x2) + (x2 - x1) * (y - y2)) / det;
        const double l1 = ((y2 - y0) * (x - x2) + (x0 - x2) * (y - y2)) / det;
        const double l2 = 1.0 - l0 - l1;
        if (l0 >= -eps && l1 >= -eps && l2 >= -eps) {
            res = l0 * val[a0] + l1 * val[a1] + l2 * val[a2];
            break;
        }
    }
    out[k] = res;
}

// Clough-Tocher split of triangle (V0, V1, V2) at its centroid C into three
// cubic Bezier patches (Farin 1986).  Control points: vertex values; next to
// each vertex along each edge, value + gradient . edge / 3; toward C, the
// average of a vertex's three points (C1 at the vertex); on each outer edge's
// middle row, the point that makes the cross-boundary derivative linear along
// the edge, in the direction from the neighbouring triangle's centroid to C
// (from the edge midpoint to C on the hull); C1 across the inner edges fixes
// the rest.  Written for one evaluation at barycentric coordinates b.
__device__ double ct_value(const double* vx, const double* vy, const double* f, const double* gx,
                           const double* gy, const double* nx, const double* ny, const bool* has_nb,
                           const double* b) {
    const double cx = (vx[0] + vx[1] + vx[2]) / 3.0, cy = (vy[0] + vy[1] + vy[2]) / 3.0;
    double e[3][3];                               // e[a][b]: control point next to a toward b
    for (int a = 0; a < 3; ++a) {
        e[a][a] = f[a];
        for (int c = 0; c < 3; ++c)
            if (c != a) e[a][c] = f[a] + (gx[a] * (vx[c] - vx[a]) + gy[a] * (vy[c] - vy[a])) / 3.0;
    }
    double inner[3], cross[3], near[3];
    for (int a = 0; a < 3; ++a)
        inner[a] = (e[a][a] + e[a][(a + 1) % 3] + e[a][(a + 2) % 3]) / 3.0;
    for (int a = 0; a < 3; ++a) {                 // outer edge a -> a+1, opposite vertex k
        const int c = (a + 1) % 3, k = 3 - a - c;
        double al = -0.5, be = -0.5;
        if (has_nb[k]) {
            // direction d = C - C_neighbour = al' (V_a - C) + be' (V_c - C); al = al'/gm, be = be'/gm,
            // gm = -(al' + be') (the weight of C)
            const double dx = cx - nx[k], dy = cy - ny[k];
            const double a00 = vx[a] - cx, a01 = vx[c] - cx, a10 = vy[a] - cy, a11 = vy[c] - cy;
            const double det = a00 * a11 - a01 * a10;
            const double p = (dx * a11 - a01 * dy) / det, q = (a00 * dy - a10 * dx) / det;
            const double gm = -(p + q);
            al = p / gm;
            be = q / gm;
        }
        const double q0 = al * e[a][a] + be * e[a][c] + inner[a];
        const double q2 = al * e[c][a] + be * e[c][c] + inner[c];
        cross[a] = (q0 + q2) / 2.0 - al * e[a][c] - be * e[c][a];
    }
    for (int a = 0; a < 3; ++a) near[a] = (inner[a] + cross[a] + cross[(a + 2) % 3]) / 3.0;
    const double center = (near[0] + near[1] + near[2]) / 3.0;
    // patch (a, c, C) opposite the smallest barycentric coordinate m
    int m = 0;
    if (b[1] < b[m]) m = 1;
    if (b[2] < b[m]) m = 2;
    const int a = (m + 1) % 3, c = (m + 2) % 3;
    const double u = b[a] - b[m], v = b[c] - b[m], w = 3.0 * b[m];
    const double cr = cross[a];
    return u * u * u * e[a][a] + 3.0 * u * u * v * e[a][c] + 3.0 * u * v * v * e[c][a] +
           v * v * v * e[c][c] + 3.0 * u * u * w * inner[a] + 6.0 * u * v * w * cr +
           3.0 * v * v * w * inner[c] + 3.0 * u * w * w * near[a] + 3.0 * v * w * w * near[c] +
           w * w * w * center;
}

__global__ void ct_kernel(const double* __restrict__ px, const double* __restrict__ py,
                          const double* __restrict__ val, const double* __restrict__ gxv,
                          const double* __restrict__ gyv, const int* __restrict__ tri,
                          const int* __restrict__ nbr, const int* __restrict__ bstart,
                          const int* __restrict__ blist, int nb, int N, double* __restrict__ out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long long)N * N) return;
    const int i = (int)(k / N), j = (int)(k % N);
    const double h = 100.0 / (N - 1);
    const double x = i * h, y = j * h;
    int bx = (int)(x / 100.0 * nb), by = (int)(y / 100.0 * nb);
    bx = min(max(bx, 0), nb - 1);
    by = min(max(by, 0), nb - 1);
    const int bk = by * nb + bx;
    double res = NAN;
    const double eps = 1e-12;
    for (int q = bstart[bk]; q < bstart[bk + 1]; ++q) {
        const int t = blist[q];
        const int a0 = tri[3 * t], a1 = tri[3 * t + 1], a2 = tri[3 * t + 2];
        const double x0 = px[a0], y0 = py[a0], x1 = px[a1], y1 = py[a1], x2 = px[a2], y2 = py[a2];
        const double det = (y1 - y2) * (x0 - x2) + (x2 - x1) * (y0 - y2);
        if (det == 0.0) continue;
        const double l0 = ((y1 - y2) * (x - x2) + (x2 - x1) * (y - y2)) / det;
        const double l1 = ((y2 - y0) * (x - x2) + (x0 - x2) * (y - y2)) / det;
        const double l2 = 1.0 - l0 - l1;
        if (l0 >= -eps && l1 >= -eps && l2 >= -eps) {
            const int iv[3] = {a0, a1, a2};
            double vx[3], vy[3], f[3], gx[3], gy[3], cnx[3], cny[3];
            bool has[3];
            for (int v = 0; v < 3; ++v) {
                vx[v] = px[iv[v]]; vy[v] = py[iv[v]]; f[v] = val[iv[v]];
                gx[v] = gxv[iv[v]]; gy[v] = gyv[iv[v]];
                const int n = nbr[3 * t + v];
                has[v] = n >= 0;
                cnx[v] = cny[v] = 0.0;
                if (has[v]) {
                    const int b0 = tri[3 * n], b1 = tri[3 * n + 1], b2 = tri[3 * n + 2];
                    cnx[v] = (px[b0] + px[b1] + px[b2]) / 3.0;
                    cny[v] = (py[b0] + py[b1] + py[b2]) / 3.0;
                }
            }
            const double bc[3] = {l0, l1, l2};
            res = ct_value(vx, vy, f, gx, gy, cnx, cny, has, bc);
            break;
        }
    }
    out[k] = res;
}

// Box-Muller pair from two Philox words
__device__ __forceinline__ void normal2(uint32_t a, uint32_t b, double* z0, double* z1) {
    const double u1 = ((double)a + 0.5) * 2.3283064365386963e-10;     // (0,1)
    const double u2 = ((double)b + 0.5) * 2.3283064365386963e-10;
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
}

__global__ void uncertainty_kernel(const double* __restrict__ mua, const double* __restrict__ mus,
                                   const double* __restrict__ rstd, const double* __restrict__ tstd,
                                   int N, int M, uint32_t k0, uint32_t k1,
                                   double* __restrict__ mua_unc, double* __restrict__ mus_unc) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long long)N * N) return;
    const int i = (int)(k / N), j = (int)(k % N);
    const double h = 100.0 / (N - 1);
    const double R = i * h, T = j * h;
    const double sR = rstd[k], sT = tstd[k];
    if (isnan(sR) || isnan(sT) || sR < 0 || sT < 0) {
        mua_unc[k] = NAN;
        mus_unc[k] = NAN;
        return;
    }
    // running mean / M2 (Welford) of the sampled table values; a NaN sample
    // makes that table's result NaN, as np.std of a list containing NaN is NaN
    double ma = 0, qa = 0, ms = 0, qs = 0;
    bool nan_a = false, nan_s = false;
    for (int d = 0; d < M; d += 2) {
        const ismc_u4 r = ismc_philox4x32_10((uint32_t)d, (uint32_t)k, (uint32_t)(k >> 32), 0x7AB1E5u,
                                              k0, k1);
        double zr[2], zt[2];
        normal2(r.x, r.y, &zr[0], &zr[1]);
        normal2(r.z, r.w, &zt[0], &zt[1]);
        for (int e = 0; e < 2 && d + e < M; ++e) {
            const int ri = nearest_idx(R + sR * zr[e], N), ti = nearest_idx(T + sT * zt[e], N);
            const double va = mua[(long long)ri * N + ti], vs = mus[(long long)ri * N + ti];
            nan_a |= isnan(va);
            nan_s |= isnan(vs);
            const double cnt = d + e + 1;
            const double da = va - ma, ds = vs - ms;
            ma += da / cnt;
            ms += ds / cnt;
            qa += da * (va - ma);
            qs += ds * (vs - ms);
        }
    }
    const double ca = mua[k], cs = mus[k];
    mua_unc[k] = nan_a ? NAN : 100.0 * sqrt(qa / M) / ca;
    mus_unc[k] = nan_s ? NAN : 100.0 * sqrt(qs / M) / cs;
}

__global__ void lookup_kernel(const double* __restrict__ table, int N, const double* __restrict__ R,
                              const double* __restrict__ T, int n, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    // lookup.py:467-489 indexes table[T_i][R_i] of the transposed table
    out[k] = table[(long long)nearest_idx(T[k], N) * N + nearest_idx(R[k], N)];
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

#define TCK(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ismc_lib_error(ISMC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// bucket grid over [0,100]^2: each triangle listed in every bucket its box touches
static int build_buckets(const double* R, const double* T, const int32_t* tri, uint32_t ntri,
                         std::vector<int>& start, std::vector<int>& list) {
    const int nb = std::max(1, std::min(256, (int)std::sqrt((double)ntri)));
    std::vector<std::vector<int>> buckets(nb * nb);
    auto cell = [&](double v) { return std::min(nb - 1, std::max(0, (int)(v / 100.0 * nb))); };
    for (uint32_t t = 0; t < ntri; ++t) {
        double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
        for (int c = 0; c < 3; ++c) {
            const int v = tri[3 * t + c];
            x0 = std::min(x0, R[v]); x1 = std::max(x1, R[v]);
            y0 = std::min(y0, T[v]); y1 = std::max(y1, T[v]);
        }
        if (x1 < 0 || y1 < 0 || x0 > 100 || y0 > 100) continue;
        for (int by = cell(y0); by <= cell(y1); ++by)
            for (int bx = cell(x0); bx <= cell(x1); ++bx) buckets[by * nb + bx].push_back((int)t);
    }
    start.assign(nb * nb + 1, 0);
    list.clear();
    for (int b = 0; b < nb * nb; ++b) {
        start[b + 1] = start[b] + (int)buckets[b].size();
        list.insert(list.end(), buckets[b].begin(), buckets[b].end());
    }
    if (list.empty()) list.push_back(0);
    return nb;
}

static int check_tri(const int32_t* tri, uint32_t ntri, uint32_t npts, const char* who) {
    for (uint32_t t = 0; t < 3 * ntri; ++t)
        if (tri[t] < 0 || (uint32_t)tri[t] >= npts)
            return ismc_lib_error(ISMC_ERR_INVALID_ARG, "%s: triangle index out of range", who);
    return 0;
}

extern "C" int ismc_table_interp(const double* R, const double* T, const double* val, uint32_t npts,
                                 const int32_t* tri, uint32_t ntri, uint32_t N, double* out) {
    if (!R || !T || !val || !tri || !out || npts < 3 || ntri == 0 || N < 2)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp: bad arguments");
    if (int rc = check_tri(tri, ntri, npts, "table_interp")) return rc;
    std::vector<int> start, list;
    const int nb = build_buckets(R, T, tri, ntri, start, list);
    DevBuf dx, dy, dv, dt, ds, dl, dout;
    const size_t cells = (size_t)N * N;
    TCK(cudaMalloc(&dx.p, npts * 8));
    TCK(cudaMalloc(&dy.p, npts * 8));
    TCK(cudaMalloc(&dv.p, npts * 8));
    TCK(cudaMalloc(&dt.p, ntri * 12));
    TCK(cudaMalloc(&ds.p, start.size() * 4));
    TCK(cudaMalloc(&dl.p, list.size() * 4));
    TCK(cudaMalloc(&dout.p, cells * 8));
    TCK(cudaMemcpy(dx.p, R, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dy.p, T, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dv.p, val, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dt.p, tri, ntri * 12, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(ds.p, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dl.p, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
    interp_kernel<<<(unsigned)((cells + 255) / 256), 256>>>(
        (const double*)dx.p, (const double*)dy.p, (const double*)dv.p, (const int*)dt.p,
        (const int*)ds.p, (const int*)dl.p, nb, (int)N, (double*)dout.p);
    TCK(cudaGetLastError());
    TCK(cudaMemcpy(out, dout.p, cells * 8, cudaMemcpyDeviceToHost));
    return 0;
}

// Vertex gradients that minimise the summed squared second derivative of the
// cubic Hermite interpolant along every edge (Nielson 1983; Renka & Cline
// 1984).  Per vertex i, with e = x_j - x_i, L = |e| over its neighbours j:
//   (sum 4 e e^T / L^3) g_i = sum (6 (y_j - y_i) - 2 e.g_j) e / L^3,
// solved in place vertex by vertex (Gauss-Seidel sweeps in vertex order)
// until the largest change of a sweep, relative to max(1, |g_i|), is < tol.
static void ct_gradients(const double* R, const double* T, const double* y, uint32_t n,
                         const std::vector<int>& ptr, const std::vector<int>& adj, int maxiter,
                         double tol, std::vector<double>& gx, std::vector<double>& gy) {
    gx.assign(n, 0.0);
    gy.assign(n, 0.0);
    for (int it = 0; it < maxiter; ++it) {
        double err = 0.0;
        for (uint32_t i = 0; i < n; ++i) {
            double q0 = 0, q1 = 0, q2 = 0, s0 = 0, s1 = 0;
            for (int p = ptr[i]; p < ptr[i + 1]; ++p) {
                const int j = adj[p];
                const double ex = R[j] - R[i], ey = T[j] - T[i];
                const double L = std::sqrt(ex * ex + ey * ey);
                const double L3 = L * L * L;
                const double df2 = -ex * gx[j] - ey * gy[j];
                q0 += 4 * ex * ex / L3;
                q1 += 4 * ex * ey / L3;
                q2 += 4 * ey * ey / L3;
                const double w = 6 * (y[i] - y[j]) - 2 * df2;
                s0 += w * ex / L3;
                s1 += w * ey / L3;
            }
            const double det = q0 * q2 - q1 * q1;
            const double r0 = (q2 * s0 - q1 * s1) / det, r1 = (-q1 * s0 + q0 * s1) / det;
            double change = std::max(std::fabs(gx[i] + r0), std::fabs(gy[i] + r1));
            gx[i] = -r0;
            gy[i] = -r1;
            change /= std::max(1.0, std::max(std::fabs(r0), std::fabs(r1)));
            err = std::max(err, change);
        }
        if (err < tol) break;
    }
}

extern "C" int ismc_table_interp_cubic(const double* R, const double* T, const double* val,
                                       uint32_t npts, const int32_t* tri, const int32_t* nbr,
                                       uint32_t ntri, const int32_t* adj_ptr, const int32_t* adj,
                                       uint32_t N, double* out) {
    if (!R || !T || !val || !tri || !nbr || !out || npts < 3 || ntri == 0 || N < 2)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: bad arguments");
    if (int rc = check_tri(tri, ntri, npts, "table_interp_cubic")) return rc;
    for (uint32_t t = 0; t < 3 * ntri; ++t)
        if (nbr[t] < -1 || nbr[t] >= (int32_t)ntri)
            return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: neighbour out of range");
    // vertex adjacency: the caller's (e.g. scipy's vertex_neighbor_vertices,
    // whose order the Gauss-Seidel sums then follow) or from the triangles
    std::vector<int> ptr, nb_list;
    if (adj_ptr && adj) {
        ptr.assign(adj_ptr, adj_ptr + npts + 1);
        if (ptr[0] != 0)
            return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: bad adjacency");
        for (uint32_t i = 0; i < npts; ++i)
            if (ptr[i + 1] < ptr[i])
                return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: bad adjacency");
        nb_list.assign(adj, adj + ptr[npts]);
        for (int v : nb_list)
            if (v < 0 || (uint32_t)v >= npts)
                return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: bad adjacency");
    } else {
        std::vector<std::vector<int>> a(npts);
        for (uint32_t t = 0; t < ntri; ++t)
            for (int c = 0; c < 3; ++c) {
                const int u = tri[3 * t + c], v = tri[3 * t + (c + 1) % 3];
                if (std::find(a[u].begin(), a[u].end(), v) == a[u].end()) a[u].push_back(v);
                if (std::find(a[v].begin(), a[v].end(), u) == a[v].end()) a[v].push_back(u);
            }
        ptr.assign(npts + 1, 0);
        for (uint32_t i = 0; i < npts; ++i) {
            ptr[i + 1] = ptr[i] + (int)a[i].size();
            nb_list.insert(nb_list.end(), a[i].begin(), a[i].end());
        }
    }
    for (uint32_t i = 0; i < npts; ++i)
        if (ptr[i + 1] == ptr[i])
            return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp_cubic: isolated point %u", i);
    std::vector<double> gx, gy;
    ct_gradients(R, T, val, npts, ptr, nb_list, 400, 1e-6, gx, gy);
    std::vector<int> start, list;
    const int nb = build_buckets(R, T, tri, ntri, start, list);
    DevBuf dx, dy, dv, dgx, dgy, dt, dn, ds, dl, dout;
    const size_t cells = (size_t)N * N;
    TCK(cudaMalloc(&dx.p, npts * 8)); TCK(cudaMalloc(&dy.p, npts * 8));
    TCK(cudaMalloc(&dv.p, npts * 8)); TCK(cudaMalloc(&dgx.p, npts * 8));
    TCK(cudaMalloc(&dgy.p, npts * 8)); TCK(cudaMalloc(&dt.p, ntri * 12));
    TCK(cudaMalloc(&dn.p, ntri * 12)); TCK(cudaMalloc(&ds.p, start.size() * 4));
    TCK(cudaMalloc(&dl.p, list.size() * 4)); TCK(cudaMalloc(&dout.p, cells * 8));
    TCK(cudaMemcpy(dx.p, R, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dy.p, T, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dv.p, val, npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dgx.p, gx.data(), npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dgy.p, gy.data(), npts * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dt.p, tri, ntri * 12, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dn.p, nbr, ntri * 12, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(ds.p, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dl.p, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
    ct_kernel<<<(unsigned)((cells + 127) / 128), 128>>>(
        (const double*)dx.p, (const double*)dy.p, (const double*)dv.p, (const double*)dgx.p,
        (const double*)dgy.p, (const int*)dt.p, (const int*)dn.p, (const int*)ds.p,
        (const int*)dl.p, nb, (int)N, (double*)dout.p);
    TCK(cudaGetLastError());
    TCK(cudaMemcpy(out, dout.p, cells * 8, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int ismc_table_uncertainty(const double* mua, const double* mus, const double* rstd,
                                      const double* tstd, uint32_t N, uint32_t M, uint64_t seed,
                                      double* mua_unc, double* mus_unc) {
    if (!mua || !mus || !rstd || !tstd || !mua_unc || !mus_unc || N < 2 || M == 0)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_uncertainty: bad arguments");
    const size_t cells = (size_t)N * N, bytes = cells * 8;
    DevBuf a, s, r, t, oa, os;
    TCK(cudaMalloc(&a.p, bytes)); TCK(cudaMalloc(&s.p, bytes));
    TCK(cudaMalloc(&r.p, bytes)); TCK(cudaMalloc(&t.p, bytes));
    TCK(cudaMalloc(&oa.p, bytes)); TCK(cudaMalloc(&os.p, bytes));
    TCK(cudaMemcpy(a.p, mua, bytes, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(s.p, mus, bytes, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(r.p, rstd, bytes, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(t.p, tstd, bytes, cudaMemcpyHostToDevice));
    uncertainty_kernel<<<(unsigned)((cells + 127) / 128), 128>>>(
        (const double*)a.p, (const double*)s.p, (const double*)r.p, (const double*)t.p, (int)N,
        (int)M, (uint32_t)seed, (uint32_t)(seed >> 32), (double*)oa.p, (double*)os.p);
    TCK(cudaGetLastError());
    TCK(cudaMemcpy(mua_unc, oa.p, bytes, cudaMemcpyDeviceToHost));
    TCK(cudaMemcpy(mus_unc, os.p, bytes, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int ismc_table_lookup(const double* table_t, uint32_t N, const double* R, const double* T,
                                 uint32_t n, double* out) {
    if (!table_t || !R || !T || !out || N < 2 || n == 0)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_lookup: bad arguments");
    const size_t tb = (size_t)N * N * 8;
    DevBuf dt, dr, dtt, dout;
    TCK(cudaMalloc(&dt.p, tb)); TCK(cudaMalloc(&dr.p, n * 8));
    TCK(cudaMalloc(&dtt.p, n * 8)); TCK(cudaMalloc(&dout.p, n * 8));
    TCK(cudaMemcpy(dt.p, table_t, tb, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dr.p, R, n * 8, cudaMemcpyHostToDevice));
    TCK(cudaMemcpy(dtt.p, T, n * 8, cudaMemcpyHostToDevice));
    lookup_kernel<<<(n + 255) / 256, 256>>>((const double*)dt.p, (int)N, (const double*)dr.p,
                                            (const double*)dtt.p, (int)n, (double*)dout.p);
    TCK(cudaGetLastError());
    TCK(cudaMemcpy(out, dout.p, n * 8, cudaMemcpyDeviceToHost));
    return 0;
}
