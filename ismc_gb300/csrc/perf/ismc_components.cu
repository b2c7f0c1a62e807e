// ismc_components.cu -- instruction cost of the propagator's building blocks.
//
// Each kernel runs one building block of an event 1024 times per thread, with a
// data dependence from one call to the next, on 608 blocks of 256 threads.
// Under ncu, smsp__inst_executed / (warps x 1024) is the block's cost in warp
// instructions per call; k_loop measures the loop and argument overhead that
// every kernel shares.  Used by ismc_gb300/perf.py (components); not part of
// the library.
#include <cstdio>
#include <cuda_runtime.h>
#include "../ismc_dev.h"
#include "../ismc_math.cuh"

#define ITERS 1024
#define BLOCKS 608
#define THREADS 256

__device__ __forceinline__ uint32_t lcg(uint32_t x) { return x * 1664525u + 1013904223u; }
__device__ __forceinline__ uint32_t tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

__global__ void k_loop(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) { x = lcg(x); acc += __uint_as_float((x >> 9) | 0x3F800000u); }
    out[tid()] = acc;
}
// one Philox4x32-10 block with the key schedule in shared memory (ismc_philox4x32_10_ev)
__global__ void k_philox(float* out, uint32_t seed) {
    __shared__ uint4 rk[5];
    if (threadIdx.x < 5) rk[threadIdx.x] = make_uint4(seed + threadIdx.x, seed * 3u, seed ^ 7u, seed + 11u);
    __syncthreads();
    uint32_t x = seed + tid();
    const uint32_t a0 = x * 77u, a1 = x ^ 0x1234u;
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) {
        x = lcg(x);
        const ismc_u4 r = ismc_philox4x32_10_ev(x, a0, a1, seed, rk);
        acc += __uint_as_float(((r.x ^ r.y ^ r.z ^ r.w) >> 9) | 0x3F800000u);
    }
    out[tid()] = acc;
}
__global__ void k_neglog(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) { x = lcg(x); acc += ismc_neglog_u32(x); }
    out[tid()] = acc;
}
__global__ void k_sincos(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) {
        x = lcg(x);
        float s, c;
        ismc_sincos_2pi(ismc_u01(x), &s, &c);
        acc += s * c;
    }
    out[tid()] = acc;
}
__global__ void k_div(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) { x = lcg(x); acc += __fdiv_rn(0.19f, ismc_u01(x) + 0.1f); }
    out[tid()] = acc;
}
__global__ void k_sqrt(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) { x = lcg(x); acc += __fsqrt_rn(ismc_u01(x)); }
    out[tid()] = acc;
}
// the division-free reflect-or-transmit draw of an interface
__global__ void k_fresnel(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float acc = 0.f;
    for (int i = 0; i < ITERS; ++i) {
        x = lcg(x);
        float ct;
        const bool r = ismc_fresnel_reflects(0.92f, ismc_u01(x), ismc_u01(x * 7u), &ct);
        acc += r ? ct : 1.f;
    }
    out[tid()] = acc;
}
// the spin of an interaction: Henyey-Greenstein cosine, azimuth, rotation
__global__ void k_spin(float* out, uint32_t seed) {
    uint32_t x = seed + tid();
    float ux = 0.3f, uy = 0.4f, uz = 0.866f;
    const float hgc = 1 - 0.81f, hgd = 0.1f, hge = 1.8f, hga = 1 / 1.8f, hgb = 1.81f;
    for (int i = 0; i < ITERS; ++i) {
        x = lcg(x);
        const float u1 = ismc_u01(x), u2 = ismc_u01(x * 2654435761u);
        const float t = __fdiv_rn(hgc, __fmaf_rn(hge, u1, hgd));
        const float cth = fminf(fmaxf(hga * __fmaf_rn(-t, t, hgb), -1.0f), 1.0f);
        float sp, cp;
        ismc_sincos_2pi(u2, &sp, &cp);
        const float s2 = fmaxf(__fmaf_rn(-cth, cth, 1.0f), 0.0f);
        if (fabsf(uz) > 0.99999f) {
            const float sth = __fsqrt_rn(s2);
            ux = sth * cp; uy = sth * sp; uz = uz > 0.0f ? cth : -cth;
        } else {
            const float rho2 = __fmaf_rn(ux, ux, uy * uy);
            const float k = __fsqrt_rn(__fdiv_rn(s2, rho2));
            const float bx = __fmaf_rn(ux * uz, cp, -(uy * sp));
            const float by = __fmaf_rn(uy * uz, cp, ux * sp);
            const float nx = __fmaf_rn(k, bx, ux * cth), ny = __fmaf_rn(k, by, uy * cth);
            const float nz = __fmaf_rn(-(k * cp), rho2, uz * cth);
            ux = nx; uy = ny; uz = nz;
        }
    }
    out[tid()] = ux + uy + uz;
}

int main() {
    float* d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * BLOCKS * THREADS) != cudaSuccess) return 1;
    k_loop<<<BLOCKS, THREADS>>>(d, 1);
    k_philox<<<BLOCKS, THREADS>>>(d, 2);
    k_neglog<<<BLOCKS, THREADS>>>(d, 3);
    k_sincos<<<BLOCKS, THREADS>>>(d, 4);
    k_div<<<BLOCKS, THREADS>>>(d, 5);
    k_sqrt<<<BLOCKS, THREADS>>>(d, 6);
    k_fresnel<<<BLOCKS, THREADS>>>(d, 7);
    k_spin<<<BLOCKS, THREADS>>>(d, 8);
    const cudaError_t e = cudaDeviceSynchronize();
    std::printf("components: %s (%d blocks x %d threads x %d calls per kernel)\n",
                cudaGetErrorString(e), BLOCKS, THREADS, ITERS);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 1;
}
