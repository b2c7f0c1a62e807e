// ismc_math.cuh -- counter-based RNG and elementary functions of the propagator.
//
// Everything here is built only from IEEE-754 single-precision operations that
// are correctly rounded on every platform (add, mul, fma, div, sqrt, int<->float
// conversion), never from hardware approximations (MUFU) or library math, and
// the translation unit is compiled with FMA contraction off so that each fma is
// written out explicitly.  A CPU restatement that performs the same operations
// in the same order therefore reproduces every packet trajectory bit for bit.
#pragma once
#include <stdint.h>

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Counter-based: the output block is a pure function of
// (counter, key), so draws are keyed by (packet id, event index) and never by
// the lane that happens to run the packet.  Replaces the per-thread curand
// XORWOW state array of CUDA/CUDAISMLMC.h:51-68 (no state, no init kernel).
// ---------------------------------------------------------------------------
#define ISMC_PHILOX_M0 0xD2511F53u
#define ISMC_PHILOX_M1 0xCD9E8D57u
#define ISMC_PHILOX_W0 0x9E3779B9u   // golden ratio
#define ISMC_PHILOX_W1 0xBB67AE85u   // sqrt(3) - 1

struct ismc_u4 { uint32_t x, y, z, w; };

__device__ __forceinline__ ismc_u4 ismc_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                      uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += ISMC_PHILOX_W0; k1 += ISMC_PHILOX_W1; }
        const uint32_t lo0 = ISMC_PHILOX_M0 * c0, hi0 = __umulhi(ISMC_PHILOX_M0, c0);
        const uint32_t lo1 = ISMC_PHILOX_M1 * c2, hi1 = __umulhi(ISMC_PHILOX_M1, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return ismc_u4{c0, c1, c2, c3};
}

// The same generator with the key schedule precomputed: rk4[q] holds the keys
// of rounds 2q and 2q+1 as (k0, k1, k0', k1'), so the per-round key additions
// become one 16-byte shared-memory load per two rounds.
__device__ __forceinline__ ismc_u4 ismc_philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2,
                                                         uint32_t c3, const uint4* rk4) {
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const uint4 kk = rk4[q];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t k0 = h ? kk.z : kk.x, k1 = h ? kk.w : kk.y;
            const uint32_t lo0 = ISMC_PHILOX_M0 * c0, hi0 = __umulhi(ISMC_PHILOX_M0, c0);
            const uint32_t lo1 = ISMC_PHILOX_M1 * c2, hi1 = __umulhi(ISMC_PHILOX_M1, c2);
            const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
            c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        }
    }
    return ismc_u4{c0, c1, c2, c3};
}

// The same block with the parts of round 0 that do not depend on the event
// index folded in ahead of time, for counters (ev, pk_lo, pk_hi, stream):
//   a0 = umulhi(M1, pk_hi) ^ pk_lo ^ k0,  a1 = M1 * pk_hi   (per packet)
//   b  = stream ^ k1                                          (per instance)
// Rounds 1-9 take their keys from rk4 as above.
__device__ __forceinline__ ismc_u4 ismc_philox4x32_10_ev(uint32_t ev, uint32_t a0, uint32_t a1,
                                                         uint32_t b, const uint4* rk4) {
    uint32_t c0 = a0, c1 = a1, c2 = __umulhi(ISMC_PHILOX_M0, ev) ^ b, c3 = ISMC_PHILOX_M0 * ev;
#pragma unroll
    for (int r = 1; r < 10; ++r) {
        const uint4 kk = rk4[r >> 1];
        const uint32_t k0 = (r & 1) ? kk.z : kk.x, k1 = (r & 1) ? kk.w : kk.y;
        const uint32_t lo0 = ISMC_PHILOX_M0 * c0, hi0 = __umulhi(ISMC_PHILOX_M0, c0);
        const uint32_t lo1 = ISMC_PHILOX_M1 * c2, hi1 = __umulhi(ISMC_PHILOX_M1, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return ismc_u4{c0, c1, c2, c3};
}

// Uniform in the open interval (0,1) with 23-bit resolution: (k + 1/2) * 2^-23,
// k = top 23 bits.  Built as [1,2) mantissa fill minus (1 - 2^-24), which is
// exact.  Never returns 0 or 1, so "u < p" has probability p for every p in
// [0,1] and a total-internal-reflection R = 1 always reflects.
__device__ __forceinline__ float ismc_u01(uint32_t x) {
    return __uint_as_float((x >> 9) | 0x3F800000u) - 0.99999994f;
}

// -ln(u) for u in (0,1], from u = x * 2^-32 with x forced odd (32-bit
// resolution keeps the exponential tail to 22.9 mean free paths).
//   ln u = e ln2 + ln m,  m in (sqrt(1/2), sqrt(2)],  f = m - 1 (exact),
//   ln m = f - f^2/2 + f^3 Q(f),
// Q a degree-7 least-squares polynomial (derivation and error check:
// fit_log_poly.py; max relative error 1.3e-7).  No division.
__device__ __forceinline__ float ismc_neglog_u32(uint32_t x) {
    const float u = __uint2float_rn(x | 1u) * 2.3283064365386963e-10f;  // 2^-32
    const uint32_t b = __float_as_uint(u);
    int e = (int)(b >> 23) - 127;
    float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
    const float f = m - 1.0f;
    float p = __fmaf_rn(f, -0.0810155869f, 0.127123073f);
    p = __fmaf_rn(f, p, -0.129722387f);
    p = __fmaf_rn(f, p, 0.142021745f);
    p = __fmaf_rn(f, p, -0.166422471f);
    p = __fmaf_rn(f, p, 0.200014681f);
    p = __fmaf_rn(f, p, -0.25000298f);
    p = __fmaf_rn(f, p, 0.333333284f);
    const float f2 = f * f;
    const float lnm = __fmaf_rn(f2, __fmaf_rn(f, p, -0.5f), f);
    const float fe = (float)e;
    // ln2 split so that fe * LN2_HI is exact for |e| < 2^8
    const float ln = __fmaf_rn(fe, 0.693145752f, __fmaf_rn(fe, 1.42860677e-06f, lnm));
    return -ln;
}

// sin and cos of 2*pi*u, u in (0,1).  v = 4u is split into a quadrant q and a
// remainder r in [-1/2, 1/2] (exact), then sin(pi r/2) and cos(pi r/2) from
// their Taylor series (truncation 2e-9 and 1e-10 on |pi r/2| <= pi/4).
__device__ __forceinline__ void ismc_sincos_2pi(float u, float* s, float* c) {
    const float v = 4.0f * u;
    const float qf = rintf(v);
    const float r = v - qf;
    const int q = ((int)qf) & 3;
    const float r2 = r * r;
    // (pi/2)^k / k! with alternating signs
    float sp = __fmaf_rn(r2, 1.60441184e-04f, -4.68175413e-03f);   // +(pi/2)^9/9!, -(pi/2)^7/7!
    sp = __fmaf_rn(r2, sp, 7.96926262e-02f);                       // +(pi/2)^5/5!
    sp = __fmaf_rn(r2, sp, -6.45964098e-01f);                      // -(pi/2)^3/3!
    sp = __fmaf_rn(r2, sp, 1.57079637f);                           // +(pi/2)
    const float sn = r * sp;
    float cp = __fmaf_rn(r2, -2.52020423e-05f, 9.19260282e-04f);   // -(pi/2)^10/10!, +(pi/2)^8/8!
    cp = __fmaf_rn(r2, cp, -2.08634808e-02f);                      // -(pi/2)^6/6!
    cp = __fmaf_rn(r2, cp, 2.53669507e-01f);                       // +(pi/2)^4/4!
    cp = __fmaf_rn(r2, cp, -1.23370055f);                          // -(pi/2)^2/2!
    const float cs = __fmaf_rn(r2, cp, 1.0f);
    // quadrant q: (sin, cos) = (sn, cs), (cs, -sn), (-sn, -cs), (-cs, sn), as selects
    const bool swap = (q & 1) != 0;
    const float so = swap ? cs : sn, co = swap ? sn : cs;
    *s = (q & 2) ? -so : so;
    *c = ((q + 1) & 2) ? -co : co;
}

// e^-x for x >= 0 (Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, then the
// Taylor series of e^-r to r^8, truncation 2e-10).  Returns 0 beyond x = 87.
__device__ __forceinline__ float ismc_expneg(float x) {
    if (!(x < 87.0f)) return 0.0f;
    const float kf = rintf(x * 1.44269502f);
    float r = __fmaf_rn(-kf, 0.693145752f, x);
    r = __fmaf_rn(-kf, 1.42860677e-06f, r);
    const float y = -r;
    float p = __fmaf_rn(y, 2.48015876e-05f, 1.98412701e-04f);   // 1/8!, 1/7!
    p = __fmaf_rn(y, p, 1.38888892e-03f);                        // 1/6!
    p = __fmaf_rn(y, p, 8.33333377e-03f);                        // 1/5!
    p = __fmaf_rn(y, p, 4.16666679e-02f);                        // 1/4!
    p = __fmaf_rn(y, p, 1.66666672e-01f);                        // 1/3!
    p = __fmaf_rn(y, p, 0.5f);
    p = __fmaf_rn(y, p, 1.0f);
    p = __fmaf_rn(y, p, 1.0f);
    const int k = (int)kf;                                       // 0 <= k <= 126
    return p * __uint_as_float((uint32_t)(127 - k) << 23);
}

// Unpolarised Fresnel reflectance for a ray crossing from index n_i to n_t,
// eta = n_i / n_t, incidence cosine ci in [0,1]; *ct receives the cosine of
// the refracted ray (0 under total internal reflection).  Algebraic form of
// the Fresnel equations (cosines only):
//   rs = (eta ci - ct)/(eta ci + ct),  rp = (eta ct - ci)/(eta ct + ci),
//   R  = (rs^2 + rp^2)/2,
// identical to the trigonometric form of MLMC.py:45-54 / ISMC.py:62-71 and
// continuous through normal incidence, where it gives ((n_i-n_t)/(n_i+n_t))^2.
__device__ __forceinline__ float ismc_fresnel(float eta, float ci, float* ct) {
    const float s2t = (eta * eta) * (1.0f - ci * ci);
    if (s2t >= 1.0f) { *ct = 0.0f; return 1.0f; }
    const float c = __fsqrt_rn(1.0f - s2t);
    const float a = eta * ci, b = eta * c;
    const float rsn = a - c, rsd = a + c, rpn = b - ci, rpd = b + ci;
    const float x = rsn * rpd, y = rpn * rsd, den = rsd * rpd;
    *ct = c;
    return __fdiv_rn(0.5f * __fmaf_rn(x, x, y * y), den * den);
}

// The reflect-or-transmit draw u < ismc_fresnel(eta, ci, ct) without the
// division: with R = N / D and D = den^2 > 0, u < R exactly when u D < N in
// real arithmetic (the rounded forms can differ only where the division's
// rounding would flip the comparison).  A total internal reflection always
// reflects, since u < 1.
__device__ __forceinline__ bool ismc_fresnel_reflects(float eta, float ci, float u, float* ct) {
    const float s2t = (eta * eta) * (1.0f - ci * ci);
    if (s2t >= 1.0f) { *ct = 0.0f; return true; }
    const float c = __fsqrt_rn(1.0f - s2t);
    const float a = eta * ci, b = eta * c;
    const float rsn = a - c, rsd = a + c, rpn = b - ci, rpd = b + ci;
    const float x = rsn * rpd, y = rpn * rsd, den = rsd * rpd;
    *ct = c;
    return u * (den * den) < 0.5f * __fmaf_rn(x, x, y * y);
}

// Fixed-point quantisation of a non-negative packet weight (scale 2^32).
__device__ __forceinline__ unsigned long long ismc_q32(float x) {
    return __float2ull_rn(x * 4294967296.0f);
}
