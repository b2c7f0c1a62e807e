// ismc_kernels.cu -- the GB300 propagator: per-instance preparation, work-queue
// prefix, and the persistent photon-packet kernel.
//
// Compiled with -fmad=false: every fused multiply-add is written explicitly,
// so each trajectory is a fixed sequence of correctly rounded IEEE operations.
//
// Reference behaviour being restated (file:line in pdcook/ISMC):
//   incidence + sphere logic ......... ISMLMC.py:112-344, ISMC.py:173-403
//   multilayer walk ................... MLMC.py:76-202 (step-to-boundary walk)
//   glass-entry series ............... ISMLMC.py:79-93
//   sphere re-incidence probability ... ISMC.py:80-81
//   port / angle acceptance tests ..... ISMC.py:196, 223-227, 244, 271-275
// The reference GPU kernel this replaces is CUDA/CUDAISMLMC.h:132-654.
#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include "ismc_dev.h"
#include "ismc_math.cuh"

#define ISMC_FULL 0xFFFFFFFFu
#define ISMC_MAX_THREADS 512
#define ISMC_NACC 15          // per-slot counters: sum[5], sumsq[5], steps, events, reinc,
                              // capped, trapped

// ============================================================================
// Float-float arithmetic (an unevaluated sum hi + lo of two floats) for the
// deterministic analytic outputs, so that FP32 hardware reaches the 1e-6
// relative agreement with an FP64 evaluation.  Dekker / Knuth error-free
// transformations; products use the exact fma residual.
// ============================================================================
struct ff { float hi, lo; };

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return ff{s, e};
}
__device__ __forceinline__ ff ff_fast(float a, float b) {   // |a| >= |b|
    const float s = a + b;
    return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff ff_from(float a) { return ff{a, 0.0f}; }
__device__ __forceinline__ ff ff_add(ff x, ff y) {
    ff s = ff_two_sum(x.hi, y.hi);
    const float e = s.lo + (x.lo + y.lo);
    return ff_fast(s.hi, e);
}
__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
__device__ __forceinline__ ff ff_mul(ff x, ff y) {
    const float p = x.hi * y.hi;
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return ff_fast(p, e);
}
__device__ __forceinline__ ff ff_div(ff x, ff y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    const ff r = ff_sub(x, ff_mul(y, ff_from(q1)));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    return ff_fast(q1, q2);
}
// normal-incidence Fresnel reflectance ((a-b)/(a+b))^2
__device__ __forceinline__ ff ff_fresnel0(float a, float b) {
    const ff num = ff_two_sum(a, -b);
    const ff den = ff_two_sum(a, b);
    const ff q = ff_div(num, den);
    return ff_mul(q, q);
}

// Incoherent stacking of a symmetric element (reflectance r, transmittance t)
// under a composite described by front/back reflectance and transmittance:
//   D = 1 - Rb r,  Rf += Tf Tb r / D,  Tf *= t / D,  Rb = r + t^2 Rb / D,  Tb *= t / D.
struct ff_stack { ff Rf, Tf, Rb, Tb; };
__device__ __forceinline__ void ff_stack_add(ff_stack& S, ff r, ff t) {
    const ff one = ff_from(1.0f);
    const ff D = ff_sub(one, ff_mul(S.Rb, r));
    const ff Rf = ff_add(S.Rf, ff_div(ff_mul(ff_mul(S.Tf, S.Tb), r), D));
    const ff Tf = ff_div(ff_mul(S.Tf, t), D);
    const ff Rb = ff_add(r, ff_div(ff_mul(ff_mul(t, t), S.Rb), D));
    const ff Tb = ff_div(ff_mul(S.Tb, t), D);
    S.Rf = Rf; S.Tf = Tf; S.Rb = Rb; S.Tb = Tb;
}
// e^-(x.hi + x.lo) = e^-x.hi * (1 - x.lo + ...), |x.lo| <= ulp(x.hi)/2
__device__ __forceinline__ ff ff_expneg(ff x) {
    const float e = ismc_expneg(x.hi);
    return ff_mul(ff_from(e), ff_two_sum(1.0f, -x.lo));
}

// ============================================================================
// Preparation: one thread per instance.
// ============================================================================
__device__ __forceinline__ bool ismc_finite(float x) { return isfinite(x); }
__device__ __forceinline__ bool ismc_finite(double x) { return isfinite(x); }

__global__ void ismc_prepare_kernel(const ismc_instance* __restrict__ in, uint32_t n_inst,
                                    DevInst* __restrict__ out, DevRange* __restrict__ range,
                                    ismc_tally* __restrict__ tally) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_inst) return;
    const ismc_instance& I = in[i];
    const ismc_stack& S = I.stack;
    const ismc_spheres& P = I.spheres;
    DevInst D;
    // ---------------------------------------------------------------- checks
    bool ok = S.L >= 1 && S.L <= ISMC_MAXL && I.mode <= ISMC_MODE_PHYSICAL;
    const uint32_t L = ok ? S.L : 1;
    for (uint32_t l = 0; l < L && ok; ++l) {
        ok = ismc_finite(S.n[l]) && S.n[l] > 0.0f && ismc_finite(S.d[l]) && S.d[l] > 0.0f &&
             ismc_finite(S.mua[l]) && S.mua[l] >= 0.0f && ismc_finite(S.mus[l]) && S.mus[l] >= 0.0f &&
             ismc_finite(S.mut[l]) && S.mut[l] >= 0.0f && ismc_finite(S.g[l]) &&
             S.g[l] >= -1.0f && S.g[l] <= 1.0f && (S.mus[l] == 0.0f || S.mut[l] > 0.0f);
    }
    double pR = 0.0, pT = 0.0, cR = 0.0, cT = 0.0;
    if (ok) {
        // sphere multiplier series in closed form, FP64: pw fs / (1 - pw (1 - f))  (ISMC.py:80-81)
        const double dR = 1.0 - P.R_pw * (1.0 - P.R_f);
        const double dT = 1.0 - P.T_pw * (1.0 - P.T_f);
        if (P.R) { ok = ok && dR > 0.0 && P.R_fp >= 0.0 && P.R_fp <= 1.0; pR = P.R_pw * P.R_fs / dR; }
        if (P.T) { ok = ok && dT > 0.0 && P.T_fp >= 0.0 && P.T_fp <= 1.0; pT = P.T_pw * P.T_fs / dT; }
        // acceptance cosines: sqrt(1 - fp) with a sphere (ISMC.py:196, 244);
        // without one fp = (1 - cos 2 angle)/2 (ISMC.py:223, 271)
        const double fpR = P.R ? P.R_fp : 0.5 * (1.0 - cos(2.0 * P.R_angle));
        const double fpT = P.T ? P.T_fp : 0.5 * (1.0 - cos(2.0 * P.T_angle));
        cR = sqrt(1.0 - fpR);
        cT = sqrt(1.0 - fpT);
        ok = ok && ismc_finite(pR) && ismc_finite(pT) && ismc_finite(cR) && ismc_finite(cT) &&
             I.roulette_m >= 1.0f && I.roulette_threshold >= 0.0f &&
             I.roulette_threshold * I.roulette_m <= 1.0f;
    }
    // 64-bit tallies at 2^-32 per unit weight: at most 2^31 packets (ismc.h)
    const bool fits = I.n_packets <= ISMC_MAX_PACKETS;
    const bool run = ok && fits;
    // ---------------------------------------------------------------- header
    D.L = L;
    D.mode = I.mode;
    D.flags = (P.R ? ISMC_IF_RSPHERE : 0u) | (P.T ? ISMC_IF_TSPHERE : 0u);
    D.stream = I.stream;
    D.seed_lo = (uint32_t)(I.seed & 0xFFFFFFFFull);
    D.seed_hi = (uint32_t)(I.seed >> 32);
    for (int r = 0; r < 10; ++r) {
        D.rk[2 * r] = D.seed_lo + (uint32_t)r * ISMC_PHILOX_W0;
        D.rk[2 * r + 1] = D.seed_hi + (uint32_t)r * ISMC_PHILOX_W1;
    }
    D.stream_k1 = D.stream ^ D.rk[1];
    D.cos_port[0] = (float)cR;
    D.cos_port[1] = (float)cT;
    D.p_reinc[0] = (float)pR;
    D.p_reinc[1] = (float)pT;
    if (P.specular_included) {      // ISMC.py:178
        D.ux0 = (float)sqrt(1.0 - 0.99 * 0.99);
        D.uz0 = 0.99f;
    } else {
        D.ux0 = 0.0f;
        D.uz0 = 1.0f;
    }
    D.roul_thr = I.roulette_threshold;
    D.roul_m = I.roulette_m;
    D.roul_inv_m = ok ? __fdiv_rn(1.0f, I.roulette_m) : 0.0f;
    D._hpad = 0u;
    // ---------------------------------------------------------------- layers
    float z = 0.0f;
    for (uint32_t l = 0; l < ISMC_MAXL; ++l) {
        const bool act = l < L;
        const float n = act ? S.n[l] : 1.0f;
        const float mut = act ? S.mut[l] : 0.0f;
        const float g = act ? S.g[l] : 0.0f;
        const bool glass = act && S.mus[l] == 0.0f;
        D.ly[l].n = n;
        D.ly[l].mut = mut;
        D.ly[l].inv_mut = mut > 0.0f ? __fdiv_rn(1.0f, mut) : 0.0f;
        D.ly[l].drop = !act ? 0.0f : (glass ? S.mua[l] : __fdiv_rn(S.mua[l], mut));
        const float g2 = 2.0f * g;
        D.ly[l].hga = g != 0.0f ? __fdiv_rn(1.0f, g2) : 0.0f;
        D.ly[l].hgb = 1.0f + g * g;
        D.ly[l].hgc = 1.0f - g * g;
        D.ly[l].hgd = 1.0f - g;
        D.ly[l].hge = g2;
        D.ly[l].z_top = z;
        if (act) z = z + S.d[l];
        D.ly[l].z_bot = z;
        const float n_above = (l == 0 || !act) ? 1.0f : S.n[l - 1];
        const float n_below = (l + 1 >= L || !act) ? 1.0f : S.n[l + 1];
        D.ly[l].eta_up = __fdiv_rn(n, n_above);
        D.ly[l].eta_dn = __fdiv_rn(n, n_below);
        D.ly[l].lflags = (glass ? ISMC_LF_GLASS : 0u) | (g == 0.0f ? ISMC_LF_ISO : 0u);
    }
    D.t_tot = z;
    D.eta_in[0] = __fdiv_rn(1.0f, S.n[0 < L ? 0 : 0]);
    D.eta_in[1] = __fdiv_rn(1.0f, S.n[L - 1]);
    // the launch's incidence on the top face, as the incidence event computes it
    {
        float ct;
        float R = ismc_fresnel(D.eta_in[0], fabsf(D.uz0), &ct);
        if (I.mode == ISMC_MODE_COMPAT && (D.ly[0].lflags & ISMC_LF_GLASS)) {
            float ct2;
            const float r2 = ismc_fresnel(D.ly[0].eta_dn, fabsf(D.uz0), &ct2);
            const float om = 1.0f - R;
            R = R + __fdiv_rn((om * om) * r2, 1.0f - R * r2);
        }
        D.launch_R = R;
        D.launch_ct = ct;
        D._hpad2[0] = D._hpad2[1] = 0u;
    }
    out[i] = D;

    // ---------------------------------------------------------------- analytic
    // (a) specular reflectance at normal incidence.  Compatible mode: the
    //     incidence series of ISMLMC.py:79-93, r1 + (1-r1)^2 r2 / (1 - r1 r2),
    //     when the top layer is a slide, else the single Fresnel term.
    //     Physical mode: the incoherent stack of every element above the first
    //     scattering layer (slides with their absorption), reflectance seen from
    //     the ambient.
    // (b) ballistic transmittance at normal incidence: the incoherent stack of
    //     every interface and layer, each layer attenuating by exp(-mut d).
    float spec = 0.0f, ball = 0.0f;
    if (ok) {
        const ff one = ff_from(1.0f), zero = ff_from(0.0f);
        if (I.mode == ISMC_MODE_COMPAT) {
            const ff r1 = ff_fresnel0(1.0f, S.n[0]);
            ff R = r1;
            if (S.mus[0] == 0.0f) {
                const ff r2 = ff_fresnel0(S.n[0], L > 1 ? S.n[1] : 1.0f);
                const ff om = ff_sub(one, r1);
                R = ff_add(r1, ff_div(ff_mul(ff_mul(om, om), r2), ff_sub(one, ff_mul(r1, r2))));
            }
            spec = R.hi + R.lo;
        }
        ff_stack A{zero, one, zero, one};
        bool spec_done = false;
        float n_prev = 1.0f;
        for (uint32_t l = 0; l < L; ++l) {
            const ff r = ff_fresnel0(n_prev, S.n[l]);
            ff_stack_add(A, r, ff_sub(one, r));
            if (S.mus[l] != 0.0f && !spec_done) {
                if (I.mode == ISMC_MODE_PHYSICAL) spec = A.Rf.hi + A.Rf.lo;
                spec_done = true;
            }
            const float p = S.mut[l] * S.d[l];
            const ff x{p, __fmaf_rn(S.mut[l], S.d[l], -p)};
            const ff a = ff_expneg(x);
            ff_stack_add(A, zero, a);
            n_prev = S.n[l];
        }
        const ff r = ff_fresnel0(n_prev, 1.0f);
        ff_stack_add(A, r, ff_sub(one, r));
        if (!spec_done && I.mode == ISMC_MODE_PHYSICAL) spec = A.Rf.hi + A.Rf.lo;
        ball = A.Tf.hi + A.Tf.lo;
    }

    // ---------------------------------------------------------------- tally / queue
    ismc_tally& T = tally[i];
    T.n = run ? I.n_packets : 0ull;
    for (int k = 0; k < 5; ++k) { T.sum[k] = 0ull; T.sumsq[k] = 0ull; }
    T.steps = T.events = T.reincidences = T.capped = T.trapped = 0ull;
    T.scale_log2 = 32u;
    T.status = !ok ? ISMC_ERR_INVALID_ARG : (fits ? ISMC_OK : ISMC_ERR_CAPACITY);
    T.analytic_specular = spec;
    T.analytic_ballistic = ball;
    const uint64_t cnt = run ? I.n_packets : 0ull;
    range[i].offset = I.packet_offset;
    range[i].count = cnt;
}

// One block: choose the packets per queue chunk from the batch's total packet
// count (so that each warp gets ~chunks_per_warp chunks and the tail stays
// short), then the inclusive prefix of per-instance chunk counts, prefix[0]=0,
// and reset of the queue head.  ctrl[0] = queue head, ctrl[1] = chunk size.
__global__ void __launch_bounds__(1024) ismc_scan_kernel(unsigned long long* prefix,
                                                         const DevRange* __restrict__ range,
                                                         uint32_t n, unsigned long long* ctrl,
                                                         uint32_t chunk_override,
                                                         uint32_t total_warps,
                                                         uint32_t chunks_per_warp) {
    __shared__ unsigned long long part[1024];
    __shared__ unsigned long long chunk_s;
    const uint32_t t = threadIdx.x;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t b = t * per, e = min(n, b + per);
    // total packets
    unsigned long long s = 0;
    for (uint32_t i = b; i < e; ++i) s += range[i].count;
    part[t] = s;
    __syncthreads();
    for (uint32_t off = blockDim.x / 2; off > 0; off >>= 1) {
        if (t < off) part[t] += part[t + off];
        __syncthreads();
    }
    if (t == 0) {
        unsigned long long c = chunk_override;
        if (c == 0) {
            const unsigned long long want = (unsigned long long)total_warps * max(chunks_per_warp, 1u);
            c = (part[0] + want - 1) / want;
            c = (c + 31) / 32 * 32;
            c = min(max(c, 32ull), 65536ull);
        }
        chunk_s = c;
    }
    __syncthreads();
    const unsigned long long chunk = chunk_s;
    // per-instance chunk counts and their inclusive scan
    s = 0;
    for (uint32_t i = b; i < e; ++i) s += (range[i].count + chunk - 1) / chunk;
    part[t] = s;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        const unsigned long long v = t >= off ? part[t - off] : 0ull;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned long long run = t ? part[t - 1] : 0ull;
    for (uint32_t i = b; i < e; ++i) {
        run += (range[i].count + chunk - 1) / chunk;
        prefix[i + 1] = run;
    }
    if (t == 0) {
        prefix[0] = 0ull;
        ctrl[0] = 0ull;
        ctrl[1] = chunk;
    }
}

// ============================================================================
// Persistent propagator.
//
// Each warp drains chunks of (instance, packet range) from a global queue and
// hands packets to its lanes as they free up: a lane whose packet ends gets the
// next packet id of the warp's current chunk at the top of the next iteration,
// so no lane idles while work is left.  A warp holds the tables of up to two
// instances in shared-memory slots (the chunk it is starting and the one its
// last packets belong to) together with per-slot integer tallies; a slot is
// flushed to the instance's global tally with 64-bit atomics when it is reused
// and when the warp retires.
//
// One iteration = one event of every live lane, and every event draws exactly
// one Philox block keyed by (event index, packet id, stream; seed).  Events:
//   INCIDENT  packet in the ambient facing the sample (launch or re-incidence)
//   WALK      packet inside layer `layer`: either reaches the next interface
//             (Fresnel reflect / refract / exit into a sphere) or interacts
//             inside the layer (hop, drop, roulette, spin, next free path).
// ============================================================================
struct WarpSlots {
    DevInst slot[2];
    unsigned long long acc[2][ISMC_NACC];
};
// the round keys are read as 16-byte words from every slot of every warp
static_assert(offsetof(DevInst, rk) % 16 == 0, "DevInst::rk alignment");
static_assert(sizeof(DevInst) % 16 == 0 && sizeof(WarpSlots) % 16 == 0, "slot alignment");

#define PH_INCIDENT 0u
#define PH_WALK 1u

__device__ __forceinline__ void ismc_flush_slot(WarpSlots* ws, int s, int inst, ismc_tally* tally,
                                                int lane) {
    if (inst >= 0 && lane < ISMC_NACC) {
        const unsigned long long v = ws->acc[s][lane];
        if (v) atomicAdd(reinterpret_cast<unsigned long long*>(&tally[inst]) + 1 + lane, v);
    }
    __syncwarp();
    if (lane < ISMC_NACC) ws->acc[s][lane] = 0ull;
    __syncwarp();
}

// A lane's step, event and re-incidence counts run up in registers across its
// packets and reach the slot's accumulators only when the lane moves to the
// other slot, when that slot is recycled, before a count could pass 2^31, and
// when the warp retires (integer sums: the order of additions is irrelevant).
__device__ __forceinline__ void ismc_flush_counts(unsigned long long* acc, uint32_t& lsteps,
                                                  uint32_t& lev, uint32_t& lreinc) {
    if (lsteps) atomicAdd(acc + 10, (unsigned long long)lsteps);
    if (lev) atomicAdd(acc + 11, (unsigned long long)lev);
    if (lreinc) atomicAdd(acc + 12, (unsigned long long)lreinc);
    lsteps = lev = lreinc = 0u;
}

__device__ __forceinline__ void ismc_load_slot(WarpSlots* ws, int s, const DevInst* src, int lane) {
    const uint32_t* g = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&ws->slot[s]);
    constexpr int W = (int)(sizeof(DevInst) / 4);
    for (int k = lane; k < W; k += 32) d[k] = __ldg(g + k);
    __syncwarp();
}

// A packet inside slide l whose direction both faces totally reflect can never
// leave.  In exact arithmetic refraction is reversible and this cannot happen;
// in FP32 it can after near-grazing entry (|mu_z| ~ 1e-4 in the previous
// layer).  Same expression as the TIR test of ismc_fresnel.
__device__ __forceinline__ bool ismc_trapped(const DevInst& I, int l, float uz) {
    const float ci = fabsf(uz);
    const float s = 1.0f - ci * ci;
    const float eu = I.ly[l].eta_up, ed = I.ly[l].eta_dn;
    return (eu * eu) * s >= 1.0f && (ed * ed) * s >= 1.0f;
}

// 16-byte word k of layer l's constants (see DevLayer)
__device__ __forceinline__ float4 ismc_lq(const DevInst& I, int l, int k) {
    return reinterpret_cast<const float4*>(&I.ly[l])[k];
}

// Branch statistics, compiled in only with -DISMC_BRANCH_STATS (a separate
// library built by ismc_gb300/perf.py, never the product): for each branch of
// the event loop, how many warp executions it had and how many lanes were
// active in them.  ismc_branch_stats[2k] counts executions of branch k,
// [2k+1] sums their active lanes.
#ifdef ISMC_BRANCH_STATS
__device__ unsigned long long ismc_branch_stats[32];
#define ISMC_BRANCH(k)                                                                   \
    do {                                                                                 \
        const unsigned m_ = __activemask();                                              \
        if ((int)(threadIdx.x & 31) == __ffs(m_) - 1) {                                  \
            atomicAdd(&ismc_branch_stats[2 * (k)], 1ull);                                \
            atomicAdd(&ismc_branch_stats[2 * (k) + 1], (unsigned long long)__popc(m_));  \
        }                                                                                \
    } while (0)
extern "C" int ismc_branch_stats_read(unsigned long long* out) {
    return cudaMemcpyFromSymbol(out, ismc_branch_stats, sizeof(ismc_branch_stats)) == cudaSuccess
               ? 0 : -1;
}
extern "C" int ismc_branch_stats_reset(void) {
    static const unsigned long long z[32] = {0};
    return cudaMemcpyToSymbol(ismc_branch_stats, z, sizeof z) == cudaSuccess ? 0 : -1;
}
#else
#define ISMC_BRANCH(k) do { } while (0)
#endif
// branch numbers of ISMC_BRANCH
enum { ISMC_BR_ITER = 0, ISMC_BR_HANDOUT, ISMC_BR_EVENT, ISMC_BR_INCIDENT, ISMC_BR_WALK,
       ISMC_BR_INTERFACE, ISMC_BR_INTERACTION, ISMC_BR_SPIN, ISMC_BR_SPHERE, ISMC_BR_FIN };

extern "C" __global__ void __launch_bounds__(ISMC_MAX_THREADS)
ismc_propagate_kernel(const PropParams P) {
    extern __shared__ __align__(16) unsigned char ismc_smem[];
    const int lane = threadIdx.x & 31;
    WarpSlots* ws = reinterpret_cast<WarpSlots*>(ismc_smem) + (threadIdx.x >> 5);
    if (lane < 2 * ISMC_NACC) (&ws->acc[0][0])[lane] = 0ull;
    __syncwarp();
    const unsigned long long n_chunks = P.chunk_prefix[P.n_inst];
    const unsigned lt_mask = (1u << lane) - 1u;

    // ---- warp-uniform queue state
    int s_inst0 = -1, s_inst1 = -1;      // instance held by slot 0 / 1
    int cur = 0;                          // slot packets are handed out from
    unsigned long long c_next = 0, c_end = 0;   // packet id range left in the current chunk
    int pend = -1;                        // claimed chunk not yet placed
    unsigned long long p_next = 0, p_end = 0;
    bool qdone = false;

    // ---- lane state
    bool alive = false;
    int slot = 0, layer = 0;
    uint32_t phase = PH_INCIDENT, side = 0;     // side 0 = R (top), 1 = T (bottom)
    uint32_t ev = 0;
    uint32_t lsteps = 0, lev = 0, lreinc = 0;   // counts not yet in a slot accumulator
    int lslot = 0;                              // the slot they belong to
    uint32_t pa0 = 0, pa1 = 0;            // the packet id's share of Philox round 0
    float w = 0.f, z = 0.f, ux = 0.f, uy = 0.f, uz = 1.f, tau = 0.f, absorbed = 0.f;

    for (;;) {
        // ================================================= hand out packets
        unsigned need = __ballot_sync(ISMC_FULL, !alive);
        ISMC_BRANCH(ISMC_BR_ITER);
        if (need) {     // every lane busy (the common case): nothing to hand out
            ISMC_BRANCH(ISMC_BR_HANDOUT);
            while (need) {
                if (c_next < c_end) {
                    const unsigned long long avail = c_end - c_next;
                    const unsigned k = (unsigned)min((unsigned long long)__popc(need), avail);
                    const unsigned rank = __popc(need & lt_mask);
                    if (!alive && rank < k) {
                        const unsigned long long id = c_next + rank;
                        const DevInst& I = ws->slot[cur];
                        alive = true;
                        slot = cur;
                        const uint32_t id_hi = (uint32_t)(id >> 32);
                        pa0 = __umulhi(ISMC_PHILOX_M1, id_hi) ^ (uint32_t)id ^ I.rk[0];
                        pa1 = ISMC_PHILOX_M1 * id_hi;
                        if (lslot != cur) {
                            ismc_flush_counts(ws->acc[lslot], lsteps, lev, lreinc);
                            lslot = cur;
                        }
                        ev = 0;
                        phase = PH_INCIDENT; side = 0;
                        w = 1.0f; absorbed = 0.0f; z = 0.0f; tau = 0.0f; layer = 0;
                        ux = I.ux0; uy = 0.0f; uz = I.uz0;
                    }
                    c_next += k;
                    need = __ballot_sync(ISMC_FULL, !alive);
                    continue;
                }
                if (pend < 0) {
                    if (qdone) break;
                    unsigned long long c = 0;
                    if (lane == 0) c = atomicAdd(P.ctrl, 1ull);
                    c = __shfl_sync(ISMC_FULL, c, 0);
                    if (c >= n_chunks) { qdone = true; break; }
                    // instance owning chunk c: last i with prefix[i] <= c
                    int inst = 0;
                    unsigned long long st = 0, en = 0;
                    if (lane == 0) {
                        uint32_t lo = 0, hi = P.n_inst;           // prefix[lo] <= c < prefix[hi]
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (P.chunk_prefix[mid] <= c) lo = mid; else hi = mid;
                        }
                        inst = (int)lo;
                        const DevRange R = P.range[lo];
                        const unsigned long long chunk_packets = P.ctrl[1];
                        const unsigned long long j = c - P.chunk_prefix[lo];
                        st = R.offset + j * chunk_packets;
                        en = R.offset + min((unsigned long long)R.count, (j + 1) * chunk_packets);
                    }
                    pend = __shfl_sync(ISMC_FULL, inst, 0);
                    p_next = __shfl_sync(ISMC_FULL, st, 0);
                    p_end = __shfl_sync(ISMC_FULL, en, 0);
                }
                // place the pending chunk into a slot
                const int cur_inst = cur ? s_inst1 : s_inst0;
                const int oth_inst = cur ? s_inst0 : s_inst1;
                if (pend == cur_inst) {
                    c_next = p_next; c_end = p_end; pend = -1;
                    continue;
                }
                if (pend == oth_inst) {
                    cur ^= 1; c_next = p_next; c_end = p_end; pend = -1;
                    continue;
                }
                const bool oth_busy = __any_sync(ISMC_FULL, alive && slot == (cur ^ 1));
                const bool cur_busy = __any_sync(ISMC_FULL, alive && slot == cur);
                int tgt = -1;
                if (!oth_busy) tgt = cur ^ 1; else if (!cur_busy) tgt = cur;
                if (tgt < 0) break;                    // both slots still draining: wait
                if (lslot == tgt) ismc_flush_counts(ws->acc[tgt], lsteps, lev, lreinc);
                __syncwarp();
                ismc_flush_slot(ws, tgt, tgt ? s_inst1 : s_inst0, P.tally, lane);
                ismc_load_slot(ws, tgt, P.inst + pend, lane);
                if (tgt) s_inst1 = pend; else s_inst0 = pend;
                cur = tgt; c_next = p_next; c_end = p_end; pend = -1;
            }
            if (!__any_sync(ISMC_FULL, alive)) {
                if (qdone && pend < 0) break;
                continue;
            }
            if (!alive) continue;
        }

        // ================================================= one event
        ISMC_BRANCH(ISMC_BR_EVENT);
        const DevInst& I = ws->slot[slot];
        const uint32_t L = I.L;
        const bool compat = I.mode == ISMC_MODE_COMPAT;
        const ismc_u4 r = ismc_philox4x32_10_ev(ev, pa0, pa1, I.stream_k1,
                                                reinterpret_cast<const uint4*>(I.rk));
        ++ev;
        const float u0 = ismc_u01(r.x);
        int fin = 0;          // 1: packet ended, 2: event cap, 3: trapped in a slide
        int bin = -1;         // tally receiving the final weight
        bool to_sphere = false;
        float c_exit = 0.0f;  // |mu_z| of the packet entering a sphere

        if (ev > P.max_events) {
            fin = 2;
        } else if (phase == PH_INCIDENT) {
            ISMC_BRANCH(ISMC_BR_INCIDENT);
            // -------- incidence on the sample (ISMLMC.py:126-229)
            const bool top = uz > 0.0f;
            const int l = top ? 0 : (int)L - 1;
            const float c = fabsf(uz);
            const float eta = I.eta_in[top ? 0 : 1];
            const bool lglass = (I.ly[l].lflags & ISMC_LF_GLASS) != 0u;
            float ct, R;
            if (ev == 1u) {
                // the launch (the packet's first event): the instance's
                // precomputed values, the same bits as computed here
                R = I.launch_R;
                ct = I.launch_ct;
            } else {
                R = ismc_fresnel(eta, c, &ct);
                if (compat && lglass) {
                    // slide on the incidence face: two-interface series with the
                    // ambient-side cosine for both interfaces (ISMLMC.py:81-91)
                    float ct2;
                    const float r2 = ismc_fresnel(top ? I.ly[l].eta_dn : I.ly[l].eta_up, c, &ct2);
                    const float om = 1.0f - R;
                    R = R + __fdiv_rn((om * om) * r2, 1.0f - R * r2);
                }
            }
            if (u0 < R) {
                to_sphere = true;
                c_exit = c;
            } else {
                ux = ux * eta;
                uy = uy * eta;
                uz = top ? ct : -ct;
                z = top ? 0.0f : I.t_tot;
                layer = l;
                phase = PH_WALK;
                tau = (compat && lglass) ? 0.0f : ismc_neglog_u32(r.w);
                if (lglass && ismc_trapped(I, l, uz)) fin = 3;
            }
        } else {
            // -------- walk inside layer l (MLMC.py:95-200)
            ISMC_BRANCH(ISMC_BR_WALK);
            const int l = layer;
            const bool down = uz > 0.0f;
            const bool glass = (I.ly[l].lflags & ISMC_LF_GLASS) != 0u;
            const float4 q0 = ismc_lq(I, l, 0);     // mut, inv_mut, drop, hgc
            const float4 q2 = ismc_lq(I, l, 2);     // z_top, z_bot, eta_up, eta_dn
            const float zb = down ? q2.y : q2.x;
            // distance to the boundary along z (rounding can leave z a hair outside)
            const float dist = fmaxf(down ? zb - z : z - zb, 0.0f);
            const float auz = fabsf(uz);
            const float mut = q0.x;
            if (glass && auz == 0.0f) {
                fin = 2;                                   // cannot leave a slide: give up on it
            } else if (glass || (auz > 0.0f && dist * mut <= tau * auz)) {
                // ---- reach the interface (free path tau/mut >= dist/|uz|, no division)
                ISMC_BRANCH(ISMC_BR_INTERFACE);
                if (!glass) {
                    const float d = __fdiv_rn(dist, auz);
                    tau = fmaxf(__fmaf_rn(-d, mut, tau), 0.0f);
                } else if (!compat && q0.z > 0.0f) {
                    const float d = __fdiv_rn(dist, auz);
                    const float wn = w * ismc_expneg(q0.z * d);
                    absorbed = absorbed + (w - wn);
                    w = wn;
                }
                z = zb;
                const int nl = down ? l + 1 : l - 1;
                const float eta = down ? q2.w : q2.z;
                float ct;
                if (ismc_fresnel_reflects(eta, auz, u0, &ct)) {
                    uz = -uz;
                } else if (nl < 0 || nl >= (int)L) {
                    side = nl < 0 ? 0u : 1u;
                    to_sphere = true;
                    c_exit = ct;
                } else {
                    ux = ux * eta;
                    uy = uy * eta;
                    uz = down ? ct : -ct;
                    // slide -> tissue leaves no path to spend: the packet
                    // interacts at the interface (MLMC.py:111, 148, 165-200)
                    const bool nglass = (I.ly[nl].lflags & ISMC_LF_GLASS) != 0u;
                    if (compat && glass && !nglass) tau = 0.0f;
                    layer = nl;
                    if (nglass && ismc_trapped(I, nl, uz)) fin = 3;
                }
            } else {
                // ---- interaction inside the layer: hop, drop, roulette, spin
                ISMC_BRANCH(ISMC_BR_INTERACTION);
                const float s = tau * q0.y;
                z = __fmaf_rn(s, uz, z);
                const float dw = w * q0.z;
                w = w - dw;
                absorbed = absorbed + dw;
                ++lsteps;
                if (w <= I.roul_thr) {                     // MLMC.py:177
                    if (u0 < I.roul_inv_m) w = w * I.roul_m;
                    else { w = 0.0f; fin = 1; }
                }
                if (!fin) {
                    ISMC_BRANCH(ISMC_BR_SPIN);
                    const float u1 = ismc_u01(r.y), u2 = ismc_u01(r.z);
                    float cth;
                    if (I.ly[l].lflags & ISMC_LF_ISO) {
                        cth = 2.0f * u1 - 1.0f;
                    } else {
                        const float4 q1 = ismc_lq(I, l, 1);     // hgd, hge, hga, hgb
                        const float t = __fdiv_rn(q0.w, __fmaf_rn(q1.y, u1, q1.x));
                        cth = q1.z * __fmaf_rn(-t, t, q1.w);
                        cth = fminf(fmaxf(cth, -1.0f), 1.0f);
                    }
                    float sp, cp;
                    ismc_sincos_2pi(u2, &sp, &cp);
                    const float s2 = fmaxf(__fmaf_rn(-cth, cth, 1.0f), 0.0f);   // sin^2 theta
                    if (fabsf(uz) > 0.99999f) {             // MLMC.py:190-193
                        const float sth = __fsqrt_rn(s2);
                        ux = sth * cp;
                        uy = sth * sp;
                        uz = uz > 0.0f ? cth : -cth;
                    } else {                                 // MLMC.py:194-198
                        // rho2 = sin^2 of the polar angle from the transverse
                        // components (= 1 - uz^2 for a unit vector; this form keeps
                        // the FP32 norm error from growing as 1/(1 - uz^2)), and
                        // k = sin(theta)/sin(polar) from one division and one root:
                        //   new = k (ux uz cp - uy sp, uy uz cp + ux sp, -rho2 cp) + cth u
                        const float rho2 = __fmaf_rn(ux, ux, uy * uy);
                        const float k = __fsqrt_rn(__fdiv_rn(s2, rho2));
                        const float bx = __fmaf_rn(ux * uz, cp, -(uy * sp));
                        const float by = __fmaf_rn(uy * uz, cp, ux * sp);
                        const float nx = __fmaf_rn(k, bx, ux * cth);
                        const float ny = __fmaf_rn(k, by, uy * cth);
                        const float nz = __fmaf_rn(-(k * cp), rho2, uz * cth);
                        ux = nx; uy = ny; uz = nz;
                    }
                    tau = ismc_neglog_u32(r.w);
                }
            }
        }

        // -------- a packet in front of a sphere port (ISMLMC.py:130-224, 239-340)
        if (to_sphere) {
            ISMC_BRANCH(ISMC_BR_SPHERE);
            const float u1 = ismc_u01(r.y);
            if (c_exit >= I.cos_port[side]) {
                bin = side ? ISMC_T_TU : ISMC_T_RS;
                fin = 1;
            } else if ((I.flags & (side ? ISMC_IF_TSPHERE : ISMC_IF_RSPHERE)) &&
                       u1 < I.p_reinc[side]) {
                // re-incident: mu_z ~ U (ISMC.py:207) or cosine-weighted sqrt(U)
                const float u2 = ismc_u01(r.z), u3 = ismc_u01(r.w);
                const float mz = compat ? u2 : __fsqrt_rn(u2);
                float sp, cp;
                ismc_sincos_2pi(u3, &sp, &cp);
                const float sn = __fsqrt_rn(__fmaf_rn(-mz, mz, 1.0f));
                ux = cp * sn;
                uy = sp * sn;
                uz = side ? -mz : mz;
                phase = PH_INCIDENT;
                ++lreinc;
            } else {
                bin = side ? ISMC_T_TD : ISMC_T_RD;
                fin = 1;
            }
        }

        if (fin) {
            ISMC_BRANCH(ISMC_BR_FIN);
            unsigned long long* acc = ws->acc[slot];
            if (fin != 2) {
                // weight absorbed so far is scored; a trapped packet's
                // remaining weight is dropped and counted
                atomicAdd(acc + ISMC_T_A, ismc_q32(absorbed));
                atomicAdd(acc + 5 + ISMC_T_A, ismc_q32(absorbed * absorbed));
                if (bin >= 0) {
                    atomicAdd(acc + bin, ismc_q32(w));
                    atomicAdd(acc + 5 + bin, ismc_q32(w * w));
                }
                if (fin == 3) atomicAdd(acc + 14, 1ull);
            } else {
                atomicAdd(acc + 13, 1ull);
                atomicMin(&P.tally[slot ? s_inst1 : s_inst0].status, ISMC_ERR_STEP_LIMIT);
            }
            lev += ev;
            if ((lev | lsteps) >= 0x80000000u) ismc_flush_counts(acc, lsteps, lev, lreinc);
            alive = false;
        }
    }
    __syncwarp();
    ismc_flush_counts(ws->acc[lslot], lsteps, lev, lreinc);
    __syncwarp();
    ismc_flush_slot(ws, 0, s_inst0, P.tally, lane);
    ismc_flush_slot(ws, 1, s_inst1, P.tally, lane);
}

// ============================================================================
// host-side launchers
// ============================================================================
int ismc_launch_prepare(const ismc_instance* d_in, uint32_t n_inst, DevInst* d_inst,
                        DevRange* d_range, unsigned long long* d_prefix, ismc_tally* d_out,
                        unsigned long long* d_ctrl, uint32_t chunk_override, uint32_t total_warps,
                        uint32_t chunks_per_warp, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (n_inst) {
        const uint32_t tb = 128;
        ismc_prepare_kernel<<<(n_inst + tb - 1) / tb, tb, 0, s>>>(d_in, n_inst, d_inst, d_range,
                                                                 d_out);
    }
    ismc_scan_kernel<<<1, 1024, 0, s>>>(d_prefix, d_range, n_inst, d_ctrl, chunk_override,
                                        total_warps, chunks_per_warp);
    return cudaGetLastError() == cudaSuccess ? 0 : ISMC_ERR_CUDA;
}

static size_t ismc_smem_bytes(uint32_t threads) { return (threads / 32) * sizeof(WarpSlots); }

int ismc_launch_propagate(const PropParams& p, uint32_t blocks, uint32_t threads, void* stream) {
    const size_t smem = ismc_smem_bytes(threads);
    static_assert(sizeof(WarpSlots) * (ISMC_MAX_THREADS / 32) <= 227 * 1024, "smem");
    cudaError_t e = cudaFuncSetAttribute(ismc_propagate_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return ISMC_ERR_CUDA;
    ismc_propagate_kernel<<<blocks, threads, smem, (cudaStream_t)stream>>>(p);
    return cudaGetLastError() == cudaSuccess ? 0 : ISMC_ERR_CUDA;
}

int ismc_propagate_occupancy(uint32_t threads, int* blocks_per_sm) {
    const size_t smem = ismc_smem_bytes(threads);
    cudaError_t e = cudaFuncSetAttribute(ismc_propagate_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return ISMC_ERR_CUDA;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, ismc_propagate_kernel,
                                                      (int)threads, smem);
    return e == cudaSuccess ? 0 : ISMC_ERR_CUDA;
}
