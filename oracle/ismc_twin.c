/*
 * ismc_twin.c -- ORACLE (test infrastructure only; never linked into the
 * product).  A CPU restatement, in FP32, of the packet-event algorithm that the
 * GPU propagator runs, with the same Philox4x32-10 stream assignment and the
 * same sequence of correctly rounded IEEE operations.  Given the same instance
 * it must produce bit-identical integer tallies, which pins the GPU kernel's
 * queue, slot, reduction and regeneration logic exactly.  Its physics is the
 * reference's (cited per block below) and is pinned separately, statistically,
 * against golden vectors produced by the reference's own Python.
 *
 * Build: see oracle/build.py (compiled with -ffp-contract=off; every fma is an
 * explicit fmaf call).
 *
 * Reference (pdcook/ISMC):
 *   driver, incidence, spheres .. ISMLMC.py:101-347, ISMC.py:164-406
 *   multilayer walk ............. MLMC.py:76-202
 *   glass incidence series ...... ISMLMC.py:79-93
 *   Fresnel ..................... MLMC.py:45-54 (restated in algebraic form)
 *   re-incidence probability .... ISMC.py:80-81
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../include/ismc.h"

/* ------------------------------------------------------------------ Philox */
static void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
}

static inline float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t b_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static inline float u01(uint32_t x) { return f_of((x >> 9) | 0x3F800000u) - 0.99999994f; }

static float neglog_u32(uint32_t x) {
    const float u = (float)(x | 1u) * 2.3283064365386963e-10f;
    const uint32_t b = b_of(u);
    int e = (int)(b >> 23) - 127;
    float m = f_of((b & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
    /* ln m = f - f^2/2 + f^3 Q(f), f = m - 1, Q degree 7 (least squares) */
    const float f = m - 1.0f;
    float p = fmaf(f, -0.0810155869f, 0.127123073f);
    p = fmaf(f, p, -0.129722387f);
    p = fmaf(f, p, 0.142021745f);
    p = fmaf(f, p, -0.166422471f);
    p = fmaf(f, p, 0.200014681f);
    p = fmaf(f, p, -0.25000298f);
    p = fmaf(f, p, 0.333333284f);
    const float f2 = f * f;
    const float lnm = fmaf(f2, fmaf(f, p, -0.5f), f);
    const float fe = (float)e;
    const float ln = fmaf(fe, 0.693145752f, fmaf(fe, 1.42860677e-06f, lnm));
    return -ln;
}

static void sincos_2pi(float u, float* s, float* c) {
    const float v = 4.0f * u;
    const float qf = rintf(v);
    const float r = v - qf;
    const int q = ((int)qf) & 3;
    const float r2 = r * r;
    float sp = fmaf(r2, 1.60441184e-04f, -4.68175413e-03f);
    sp = fmaf(r2, sp, 7.96926262e-02f);
    sp = fmaf(r2, sp, -6.45964098e-01f);
    sp = fmaf(r2, sp, 1.57079637f);
    const float sn = r * sp;
    float cp = fmaf(r2, -2.52020423e-05f, 9.19260282e-04f);
    cp = fmaf(r2, cp, -2.08634808e-02f);
    cp = fmaf(r2, cp, 2.53669507e-01f);
    cp = fmaf(r2, cp, -1.23370055f);
    const float cs = fmaf(r2, cp, 1.0f);
    switch (q) {
        case 0: *s = sn;  *c = cs;  break;
        case 1: *s = cs;  *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

static float expneg(float x) {
    if (!(x < 87.0f)) return 0.0f;
    const float kf = rintf(x * 1.44269502f);
    float r = fmaf(-kf, 0.693145752f, x);
    r = fmaf(-kf, 1.42860677e-06f, r);
    const float y = -r;
    float p = fmaf(y, 2.48015876e-05f, 1.98412701e-04f);
    p = fmaf(y, p, 1.38888892e-03f);
    p = fmaf(y, p, 8.33333377e-03f);
    p = fmaf(y, p, 4.16666679e-02f);
    p = fmaf(y, p, 1.66666672e-01f);
    p = fmaf(y, p, 0.5f);
    p = fmaf(y, p, 1.0f);
    p = fmaf(y, p, 1.0f);
    const int k = (int)kf;
    return p * f_of((uint32_t)(127 - k) << 23);
}

/* Fresnel reflectance, algebraic form; *ct = cosine of the refracted ray. */
static float fresnel(float eta, float ci, float* ct) {
    const float s2t = (eta * eta) * (1.0f - ci * ci);
    if (s2t >= 1.0f) { *ct = 0.0f; return 1.0f; }
    const float c = sqrtf(1.0f - s2t);
    const float a = eta * ci, b = eta * c;
    const float rsn = a - c, rsd = a + c, rpn = b - ci, rpd = b + ci;
    const float x = rsn * rpd, y = rpn * rsd, den = rsd * rpd;
    *ct = c;
    return (0.5f * fmaf(x, x, y * y)) / (den * den);
}

/* The draw u < fresnel(eta, ci, ct) without the division, as the GPU takes
 * it at an interface: u * den^2 < (x^2 + y^2) / 2. */
static int fresnel_reflects(float eta, float ci, float u, float* ct) {
    const float s2t = (eta * eta) * (1.0f - ci * ci);
    if (s2t >= 1.0f) { *ct = 0.0f; return 1; }
    const float c = sqrtf(1.0f - s2t);
    const float a = eta * ci, b = eta * c;
    const float rsn = a - c, rsd = a + c, rpn = b - ci, rpd = b + ci;
    const float x = rsn * rpd, y = rpn * rsd, den = rsd * rpd;
    *ct = c;
    return u * (den * den) < 0.5f * fmaf(x, x, y * y);
}

static inline uint64_t q32(float x) { return (uint64_t)llrintf(x * 4294967296.0f); }

/* ------------------------------------------------------------ instance prep */
typedef struct {
    uint32_t L, mode, rs, ts, stream, seed_lo, seed_hi;
    float t_tot, cos_port[2], p_reinc[2], ux0, uz0, thr, m, inv_m, eta_in[2];
    float n[ISMC_MAXL], mut[ISMC_MAXL], inv_mut[ISMC_MAXL], drop[ISMC_MAXL];
    float hga[ISMC_MAXL], hgb[ISMC_MAXL], hgc[ISMC_MAXL], hgd[ISMC_MAXL], hge[ISMC_MAXL];
    float z_top[ISMC_MAXL], z_bot[ISMC_MAXL], eta_up[ISMC_MAXL], eta_dn[ISMC_MAXL];
    int glass[ISMC_MAXL], iso[ISMC_MAXL];
} TwinInst;

static void prepare(const ismc_instance* I, TwinInst* D) {
    const ismc_stack* S = &I->stack;
    const ismc_spheres* P = &I->spheres;
    memset(D, 0, sizeof(*D));
    const uint32_t L = S->L;
    D->L = L;
    D->mode = I->mode;
    D->rs = P->R; D->ts = P->T;
    D->stream = I->stream;
    D->seed_lo = (uint32_t)(I->seed & 0xFFFFFFFFull);
    D->seed_hi = (uint32_t)(I->seed >> 32);
    const double fpR = P->R ? P->R_fp : 0.5 * (1.0 - cos(2.0 * P->R_angle));
    const double fpT = P->T ? P->T_fp : 0.5 * (1.0 - cos(2.0 * P->T_angle));
    D->cos_port[0] = (float)sqrt(1.0 - fpR);
    D->cos_port[1] = (float)sqrt(1.0 - fpT);
    D->p_reinc[0] = P->R ? (float)(P->R_pw * P->R_fs / (1.0 - P->R_pw * (1.0 - P->R_f))) : 0.0f;
    D->p_reinc[1] = P->T ? (float)(P->T_pw * P->T_fs / (1.0 - P->T_pw * (1.0 - P->T_f))) : 0.0f;
    if (P->specular_included) { D->ux0 = (float)sqrt(1.0 - 0.99 * 0.99); D->uz0 = 0.99f; }
    else { D->ux0 = 0.0f; D->uz0 = 1.0f; }
    D->thr = I->roulette_threshold;
    D->m = I->roulette_m;
    D->inv_m = 1.0f / I->roulette_m;
    float z = 0.0f;
    for (uint32_t l = 0; l < L; ++l) {
        const float n = S->n[l], mut = S->mut[l], g = S->g[l];
        const int glass = S->mus[l] == 0.0f;
        D->n[l] = n;
        D->mut[l] = mut;
        D->inv_mut[l] = mut > 0.0f ? 1.0f / mut : 0.0f;
        D->drop[l] = glass ? S->mua[l] : S->mua[l] / mut;
        const float g2 = 2.0f * g;
        D->hga[l] = g != 0.0f ? 1.0f / g2 : 0.0f;
        D->hgb[l] = 1.0f + g * g;
        D->hgc[l] = 1.0f - g * g;
        D->hgd[l] = 1.0f - g;
        D->hge[l] = g2;
        D->z_top[l] = z;
        z = z + S->d[l];
        D->z_bot[l] = z;
        const float na = l == 0 ? 1.0f : S->n[l - 1];
        const float nb = l + 1 >= L ? 1.0f : S->n[l + 1];
        D->eta_up[l] = n / na;
        D->eta_dn[l] = n / nb;
        D->glass[l] = glass;
        D->iso[l] = g == 0.0f;
    }
    D->t_tot = z;
    D->eta_in[0] = 1.0f / S->n[0];
    D->eta_in[1] = 1.0f / S->n[L - 1];
}

/* A slide that totally reflects the direction on both faces cannot be left;
 * only rounding at near-grazing entry produces this.  Same test as fresnel(). */
static int trapped_in(const TwinInst* I, int l, float uz) {
    const float ci = fabsf(uz);
    const float s = 1.0f - ci * ci;
    const float eu = I->eta_up[l], ed = I->eta_dn[l];
    return (eu * eu) * s >= 1.0f && (ed * ed) * s >= 1.0f;
}

/* ------------------------------------------------------------ one packet */
typedef struct {
    float absorbed, w;
    int bin;            /* tally of the final weight, -1 none */
    int capped, trapped;
    uint32_t steps, events, reinc;
} TwinPacket;

static void run_packet(const TwinInst* I, uint64_t id, uint32_t max_events, TwinPacket* o) {
    const int compat = I->mode == ISMC_MODE_COMPAT;
    uint32_t ev = 0, steps = 0, reinc = 0;
    int incident = 1, side = 0, layer = 0;
    float w = 1.0f, absorbed = 0.0f, z = 0.0f, tau = 0.0f;
    float ux = I->ux0, uy = 0.0f, uz = I->uz0;
    int bin = -1, fin = 0;
    while (!fin) {
        uint32_t r[4] = {ev, (uint32_t)id, (uint32_t)(id >> 32), I->stream};
        philox10(r, I->seed_lo, I->seed_hi);
        ++ev;
        const float u0 = u01(r[0]);
        int to_sphere = 0;
        float c_exit = 0.0f;
        if (ev > max_events) {
            fin = 2;
        } else if (incident) {
            /* incidence on the sample (ISMLMC.py:126-229) */
            const int top = uz > 0.0f;
            const int l = top ? 0 : (int)I->L - 1;
            const float c = fabsf(uz);
            const float eta = I->eta_in[top ? 0 : 1];
            float ct, ct2;
            float R = fresnel(eta, c, &ct);
            if (compat && I->glass[l]) {
                /* ISMLMC.py:81-91: r1 + (1-r1)^2 r2 / (1 - r1 r2), same cosine */
                const float r2 = fresnel(top ? I->eta_dn[l] : I->eta_up[l], c, &ct2);
                const float om = 1.0f - R;
                R = R + ((om * om) * r2) / (1.0f - R * r2);
            }
            if (u0 < R) {
                to_sphere = 1;
                c_exit = c;
            } else {
                ux = ux * eta;
                uy = uy * eta;
                uz = top ? ct : -ct;
                z = top ? 0.0f : I->t_tot;
                layer = l;
                incident = 0;
                tau = (compat && I->glass[l]) ? 0.0f : neglog_u32(r[3]);
                if (I->glass[l] && trapped_in(I, l, uz)) fin = 3;
            }
        } else {
            /* walk (MLMC.py:95-200) */
            const int l = layer;
            const int down = uz > 0.0f;
            const int glass = I->glass[l];
            const float zb = down ? I->z_bot[l] : I->z_top[l];
            const float dist = fmaxf(down ? zb - z : z - zb, 0.0f);
            const float auz = fabsf(uz);
            const float mut = I->mut[l];
            if (glass && auz == 0.0f) {
                fin = 2;
            } else if (glass || (auz > 0.0f && dist * mut <= tau * auz)) {
                /* the free path tau/mut reaches the boundary at dist/|uz| */
                if (!glass) {
                    const float d = dist / auz;
                    tau = fmaxf(fmaf(-d, mut, tau), 0.0f);
                } else if (!compat && I->drop[l] > 0.0f) {
                    const float d = dist / auz;
                    const float wn = w * expneg(I->drop[l] * d);
                    absorbed = absorbed + (w - wn);
                    w = wn;
                }
                z = zb;
                const int nl = down ? l + 1 : l - 1;
                const float eta = down ? I->eta_dn[l] : I->eta_up[l];
                float ct;
                if (fresnel_reflects(eta, auz, u0, &ct)) {
                    uz = -uz;
                } else if (nl < 0 || nl >= (int)I->L) {
                    side = nl < 0 ? 0 : 1;
                    to_sphere = 1;
                    c_exit = ct;
                } else {
                    ux = ux * eta;
                    uy = uy * eta;
                    uz = down ? ct : -ct;
                    if (compat && glass && !I->glass[nl]) tau = 0.0f;
                    layer = nl;
                    if (I->glass[nl] && trapped_in(I, nl, uz)) fin = 3;
                }
            } else {
                const float s = tau * I->inv_mut[l];
                z = fmaf(s, uz, z);
                const float dw = w * I->drop[l];
                w = w - dw;
                absorbed = absorbed + dw;
                ++steps;
                if (w <= I->thr) {
                    if (u0 < I->inv_m) w = w * I->m;
                    else { w = 0.0f; fin = 1; }
                }
                if (!fin) {
                    const float u1 = u01(r[1]), u2 = u01(r[2]);
                    float cth;
                    if (I->iso[l]) {
                        cth = 2.0f * u1 - 1.0f;
                    } else {
                        const float t = I->hgc[l] / fmaf(I->hge[l], u1, I->hgd[l]);
                        cth = I->hga[l] * fmaf(-t, t, I->hgb[l]);
                        cth = fminf(fmaxf(cth, -1.0f), 1.0f);
                    }
                    float sp, cp;
                    sincos_2pi(u2, &sp, &cp);
                    const float s2 = fmaxf(fmaf(-cth, cth, 1.0f), 0.0f);
                    if (fabsf(uz) > 0.99999f) {
                        const float sth = sqrtf(s2);
                        ux = sth * cp;
                        uy = sth * sp;
                        uz = uz > 0.0f ? cth : -cth;
                    } else {
                        /* rho2 = ux^2 + uy^2 (= 1 - uz^2 for a unit vector),
                         * k = sin(theta) / sqrt(rho2) */
                        const float rho2 = fmaf(ux, ux, uy * uy);
                        const float k = sqrtf(s2 / rho2);
                        const float bx = fmaf(ux * uz, cp, -(uy * sp));
                        const float by = fmaf(uy * uz, cp, ux * sp);
                        const float nx = fmaf(k, bx, ux * cth);
                        const float ny = fmaf(k, by, uy * cth);
                        const float nz = fmaf(-(k * cp), rho2, uz * cth);
                        ux = nx; uy = ny; uz = nz;
                    }
                    tau = neglog_u32(r[3]);
                }
            }
        }
        if (to_sphere) {
            /* sphere port / re-incidence (ISMLMC.py:130-224, 239-340) */
            const float u1 = u01(r[1]);
            if (c_exit >= I->cos_port[side]) {
                bin = side ? ISMC_T_TU : ISMC_T_RS;
                fin = 1;
            } else if ((side ? I->ts : I->rs) && u1 < I->p_reinc[side]) {
                const float u2 = u01(r[2]), u3 = u01(r[3]);
                const float mz = compat ? u2 : sqrtf(u2);
                float sp, cp;
                sincos_2pi(u3, &sp, &cp);
                const float sn = sqrtf(fmaf(-mz, mz, 1.0f));
                ux = cp * sn;
                uy = sp * sn;
                uz = side ? -mz : mz;
                incident = 1;
                ++reinc;
            } else {
                bin = side ? ISMC_T_TD : ISMC_T_RD;
                fin = 1;
            }
        }
    }
    o->absorbed = absorbed;
    o->w = w;
    o->bin = fin == 1 ? bin : -1;
    o->capped = fin == 2;
    o->trapped = fin == 3;
    o->steps = steps;
    o->events = ev;
    o->reinc = reinc;
}

/* ------------------------------------------------------------ public */
typedef struct {
    const TwinInst* I;
    uint64_t first, count;
    uint32_t max_events;
    ismc_tally t;
} Work;

static void add_packet(ismc_tally* t, const TwinPacket* p) {
    if (p->capped) {
        t->capped += 1;
    } else {
        t->sum[ISMC_T_A] += q32(p->absorbed);
        t->sumsq[ISMC_T_A] += q32(p->absorbed * p->absorbed);
        if (p->bin >= 0) {
            t->sum[p->bin] += q32(p->w);
            t->sumsq[p->bin] += q32(p->w * p->w);
        }
        if (p->trapped) t->trapped += 1;
    }
    t->steps += p->steps;
    t->events += p->events;
    t->reincidences += p->reinc;
}

static void* work_fn(void* arg) {
    Work* w = (Work*)arg;
    TwinPacket p;
    for (uint64_t k = 0; k < w->count; ++k) {
        run_packet(w->I, w->first + k, w->max_events, &p);
        add_packet(&w->t, &p);
    }
    return NULL;
}

/* Simulate one instance on `threads` host threads; integer tallies are summed,
 * so the result does not depend on the thread count. */
int twin_run(const ismc_instance* inst, uint32_t max_events, int threads, ismc_tally* out) {
    if (!inst || !out || inst->stack.L < 1 || inst->stack.L > ISMC_MAXL) return -1;
    if (inst->n_packets > ISMC_MAX_PACKETS) return -1;
    TwinInst I;
    prepare(inst, &I);
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    Work w[256];
    pthread_t th[256];
    const uint64_t n = inst->n_packets;
    for (int k = 0; k < threads; ++k) {
        memset(&w[k], 0, sizeof(Work));
        w[k].I = &I;
        w[k].first = inst->packet_offset + n * (uint64_t)k / (uint64_t)threads;
        w[k].count = inst->packet_offset + n * (uint64_t)(k + 1) / (uint64_t)threads - w[k].first;
        w[k].max_events = max_events ? max_events : 10000000u;
        pthread_create(&th[k], NULL, work_fn, &w[k]);
    }
    memset(out, 0, sizeof(*out));
    for (int k = 0; k < threads; ++k) {
        pthread_join(th[k], NULL);
        for (int j = 0; j < 5; ++j) { out->sum[j] += w[k].t.sum[j]; out->sumsq[j] += w[k].t.sumsq[j]; }
        out->steps += w[k].t.steps;
        out->events += w[k].t.events;
        out->reincidences += w[k].t.reincidences;
        out->capped += w[k].t.capped;
        out->trapped += w[k].t.trapped;
    }
    out->n = n;
    out->scale_log2 = 32;
    out->status = out->capped ? ISMC_ERR_STEP_LIMIT : ISMC_OK;
    return 0;
}

/* One packet's outcome, for trajectory-level debugging. */
int twin_packet(const ismc_instance* inst, uint64_t id, uint32_t max_events, float* absorbed,
                float* w, int* bin, uint32_t* events) {
    TwinInst I;
    TwinPacket p;
    prepare(inst, &I);
    run_packet(&I, id, max_events ? max_events : 10000000u, &p);
    *absorbed = p.absorbed; *w = p.w; *bin = p.bin; *events = p.events;
    return p.capped;
}

/* Exposed elementary functions and the raw Philox block, for unit tests. */
void twin_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox10(c, k0, k1);
    memcpy(out, c, 16);
}
float twin_u01(uint32_t x) { return u01(x); }
float twin_neglog_u32(uint32_t x) { return neglog_u32(x); }
void twin_sincos_2pi(float u, float* s, float* c) { sincos_2pi(u, s, c); }
float twin_expneg(float x) { return expneg(x); }
float twin_fresnel(float eta, float ci, float* ct) { return fresnel(eta, ci, ct); }
int twin_fresnel_reflects(float eta, float ci, float u, float* ct) {
    return fresnel_reflects(eta, ci, u, ct);
}
