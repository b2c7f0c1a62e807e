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

extern "C" int ismc_table_interp(const double* R, const double* T, const double* val, uint32_t npts,
                                 const int32_t* tri, uint32_t ntri, uint32_t N, double* out) {
    if (!R || !T || !val || !tri || !out || npts < 3 || ntri == 0 || N < 2)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp: bad arguments");
    for (uint32_t t = 0; t < 3 * ntri; ++t)
        if (tri[t] < 0 || (uint32_t)tri[t] >= npts)
            return ismc_lib_error(ISMC_ERR_INVALID_ARG, "table_interp: triangle index out of range");
    // bucket grid over [0,100]^2: each triangle listed in every bucket its box touches
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
    std::vector<int> start(nb * nb + 1, 0), list;
    for (int b = 0; b < nb * nb; ++b) {
        start[b + 1] = start[b] + (int)buckets[b].size();
        list.insert(list.end(), buckets[b].begin(), buckets[b].end());
    }
    if (list.empty()) list.push_back(0);
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
