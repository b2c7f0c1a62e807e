/*
 * ismc_ref64.c -- ORACLE (test infrastructure and CPU baseline only; never part
 * of the product).  A direct FP64 restatement of the reference's Python forward
 * model, structure for structure:
 *
 *   ref_fresnel_snell ...... ISMC.py:62-71 / MLMC.py:45-54 (trigonometric form)
 *   ref_snell .............. ISMC.py:56-59 / MLMC.py:39-42
 *   ref_incident_reflect ... ISMC.py:74-76 (single slab), ISMLMC.py:79-93 (stack)
 *   ref_reincidence ........ ISMC.py:80-81
 *   ref_mc_single .......... ISMC.py:87-160  (slab walk, mirror boundaries)
 *   ref_mc_multi ........... MLMC.py:76-202  (multilayer step-to-boundary walk)
 *   ref_mc_multi_physical .. the same walk in the kernel's physical mode (no
 *                            counterpart in the reference)
 *   ref_driver ............. ISMC.py:164-406 / ISMLMC.py:101-347
 *
 * Random numbers: the reference draws Python `random.uniform(0,1)` (Mersenne
 * Twister) sequentially; here each packet owns a Philox4x32-10 stream keyed by
 * (seed; packet id, stream) and consumes it sequentially, 53-bit uniforms in
 * [0,1).  Results therefore agree with the reference statistically, not bit for
 * bit.  Per packet the sums of each tally and of its square are returned so
 * that means and standard errors can be formed exactly as for the GPU path.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../include/ismc.h"

typedef struct {
    uint32_t k0, k1, c1, c2, c3;
    uint32_t block;
    uint32_t buf[4];
    int idx;
} Rng;

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

static uint32_t next32(Rng* g) {
    if (g->idx == 4) {
        uint32_t c[4] = {g->block++, g->c1, g->c2, g->c3};
        philox10(c, g->k0, g->k1);
        memcpy(g->buf, c, 16);
        g->idx = 0;
    }
    return g->buf[g->idx++];
}

/* random.uniform(0,1): [0,1) with 53 random bits */
static double uniform(Rng* g) {
    const uint32_t a = next32(g) >> 5, b = next32(g) >> 6;
    return ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
}

static double ref_fresnel_snell(double ni, double nt, double mu_z) {
    double R;
    if (fabs(mu_z) > 0.99999) {
        R = ((nt - ni) / (nt + ni)) * ((nt - ni) / (nt + ni));
    } else {
        const double ti = acos(fabs(mu_z));
        if ((ni * sin(ti)) / nt >= 1.0) {
            R = 1.0;
        } else {
            const double tt = asin((ni * sin(ti)) / nt);
            const double a = sin(ti - tt), b = sin(ti + tt), c = tan(ti - tt), d = tan(ti + tt);
            R = 0.5 * ((a * a) / (b * b) + (c * c) / (d * d));
        }
    }
    return R;
}

static void ref_snell(double ni, double nt, double* ux, double* uy, double* uz) {
    const double ti = acos(fabs(*uz));
    const double tt = asin((ni * sin(ti)) / nt);
    *ux = *ux * ni / nt;
    *uy = *uy * ni / nt;
    *uz = (*uz / fabs(*uz)) * cos(tt);
}

typedef struct {
    int L;
    double n[ISMC_MAXL], mua[ISMC_MAXL], mus[ISMC_MAXL], mut[ISMC_MAXL], g[ISMC_MAXL], t[ISMC_MAXL];
    double bounds[ISMC_MAXL + 1];
} Stack;

typedef struct { double absorbed, reflected, transmitted, ux, uy, uz; uint64_t steps; } Walk;

/* ISMC.py:87-160 */
/* Henyey-Greenstein deflection and azimuth, and the direction rotation with
 * its normal-incidence branch (MLMC.py:187-200) */
static void ref_spin(double gg, Rng* g, double* ux, double* uy, double* uz) {
    double ct;
    if (gg == 0.0) ct = 2 * uniform(g) - 1;
    else {
        const double q = (1 - gg * gg) / (1 - gg + 2 * gg * uniform(g));
        ct = (1 / (2 * gg)) * (1 + gg * gg - q * q);
    }
    const double phi = 2 * M_PI * uniform(g);
    const double cp = cos(phi), sp = sin(phi);
    const double st = sqrt(1.0 - ct * ct);
    double nx, ny, nz;
    if (fabs(*uz) > 0.99999) {
        nx = st * cp; ny = st * sp; nz = (*uz / fabs(*uz)) * ct;
    } else {
        const double zs = sqrt(1 - *uz * *uz);
        nx = st / zs * (*ux * *uz * cp - *uy * sp) + *ux * ct;
        ny = st / zs * (*uy * *uz * cp + *ux * sp) + *uy * ct;
        nz = -1.0 * st * cp * zs + *uz * ct;
    }
    *ux = nx; *uy = ny; *uz = nz;
}

static void ref_mc_single(const Stack* S, double w, double z, double ux, double uy, double uz,
                          Rng* g, Walk* o) {
    const double n = S->n[0], mua = S->mua[0], mut = S->mut[0], gg = S->g[0], t = S->t[0];
    double A = 0, Rf = 0, Tr = 0;
    o->steps = 0;
    while (w > 0) {
        double u = uniform(g);
        if (u <= 0) u = 1e-300;
        const double s = -log(u) / mut;
        z += s * uz;
        ++o->steps;
        while (z > t || z < 0) {
            if (z > t) {
                if (uniform(g) < ref_fresnel_snell(n, 1.0, uz)) { z = 2 * t - z; uz *= -1; }
                else { Tr += w; ref_snell(n, 1.0, &ux, &uy, &uz); w = 0; break; }
            } else if (z < 0) {
                if (uniform(g) < ref_fresnel_snell(n, 1.0, uz)) { z *= -1; uz *= -1; }
                else { Rf += w; ref_snell(n, 1.0, &ux, &uy, &uz); w = 0; break; }
            }
        }
        const double dW = w * mua / mut;
        w -= dW;
        A += dW;
        if (w <= 0.001) w = (uniform(g) <= 1.0 / 10) ? 10 * w : 0;
        if (w > 0) {
            double ct;
            if (gg == 0.0) ct = 2 * uniform(g) - 1;
            else {
                const double q = (1 - gg * gg) / (1 - gg + 2 * gg * uniform(g));
                ct = (1 / (2 * gg)) * (1 + gg * gg - q * q);
            }
            const double phi = 2 * M_PI * uniform(g);
            const double cp = cos(phi), sp = sin(phi);
            const double st = sqrt(1.0 - ct * ct);
            double nx, ny, nz;
            if (fabs(uz) > 0.99999) {
                nx = st * cp; ny = st * sp; nz = (uz / fabs(uz)) * ct;
            } else {
                const double zs = sqrt(1 - uz * uz);
                nx = st / zs * (ux * uz * cp - uy * sp) + ux * ct;
                ny = st / zs * (uy * uz * cp + ux * sp) + uy * ct;
                nz = -1.0 * st * cp * zs + uz * ct;
            }
            ux = nx; uy = ny; uz = nz;
        }
    }
    o->absorbed = A; o->reflected = Rf; o->transmitted = Tr; o->ux = ux; o->uy = uy; o->uz = uz;
}

/* MLMC.py:76-202 */
static void ref_mc_multi(const Stack* S, double w, double z, double ux, double uy, double uz,
                         Rng* g, double threshold, double m, Walk* o) {
    double A = 0, Rf = 0, Tr = 0, s = 0, d = 0;
    int layer = uz > 0 ? 0 : S->L - 1, next = layer;
    uint64_t events = 0;
    o->steps = 0;
    while (w > 0) {
        if (S->mus[layer] != 0) {
            double u = uniform(g);
            if (u <= 0) u = 1e-300;
            s = -log(u) / S->mut[layer];
            ++o->steps;
        }
        if (uz < 0) { d = (S->bounds[layer] - z) / uz; next = layer - 1; }
        else if (uz > 0) { d = (S->bounds[layer + 1] - z) / uz; next = layer + 1; }
        else { d = INFINITY; next = layer; }
        if (S->mus[layer] == 0) s = d;
        while (s >= d) {
            if (++events > 100000000ull) { w = 0; break; }   /* guard: MLMC.py has none */
            /* x, y positions are not observable: only z is tracked */
            z += d * uz;
            s -= d;
            if (next == S->L) {
                if (uniform(g) < ref_fresnel_snell(S->n[layer], 1.0, uz)) uz *= -1;
                else { Tr += w; ref_snell(S->n[layer], 1.0, &ux, &uy, &uz); w = 0; break; }
            } else if (next == -1) {
                if (uniform(g) < ref_fresnel_snell(S->n[layer], 1.0, uz)) uz *= -1;
                else { Rf += w; ref_snell(S->n[layer], 1.0, &ux, &uy, &uz); w = 0; break; }
            } else {
                if (uniform(g) < ref_fresnel_snell(S->n[layer], S->n[next], uz)) {
                    uz *= -1;
                } else {
                    ref_snell(S->n[layer], S->n[next], &ux, &uy, &uz);
                    if (S->mus[next] != 0 && s != 0) s *= S->mut[layer] / S->mut[next];
                    layer = next;
                }
            }
            if (uz < 0) { d = (S->bounds[layer] - z) / uz; next = layer - 1; }
            else if (uz > 0) { d = (S->bounds[layer + 1] - z) / uz; next = layer + 1; }
            else { d = INFINITY; next = layer; }
            if (S->mus[layer] == 0) s = d;
        }
        z += s * uz;
        if (S->mus[layer] != 0) {
            const double dW = w * S->mua[layer] / S->mut[layer];
            w -= dW;
            A += dW;
        }
        if (w <= threshold) w = (uniform(g) <= 1.0 / m) ? m * w : 0;
        if (w > 0 && S->mus[layer] != 0) ref_spin(S->g[layer], g, &ux, &uy, &uz);
    }
    o->absorbed = A; o->reflected = Rf; o->transmitted = Tr; o->ux = ux; o->uy = uy; o->uz = uz;
}

/*
 * Physical mode (no counterpart in the reference; the kernel's mode
 * ISMC_MODE_PHYSICAL).  Same step-to-boundary walk, except that
 *   - the free path is carried as optical depth tau, so what is left when a
 *     packet leaves a scattering layer survives a slide and is spent in the
 *     next scattering layer (the compat walk restarts with s = 0 there);
 *   - a slide absorbs by Beer-Lambert, w *= exp(-mua d), over the path d
 *     inside it (the compat walk ignores slide mua);
 *   - the first tau is drawn by the caller at incidence, even under a slide.
 */
static void ref_mc_multi_physical(const Stack* S, double w, double z, double ux, double uy,
                                  double uz, double tau, Rng* g, double threshold, double m,
                                  Walk* o) {
    double A = 0, Rf = 0, Tr = 0;
    int layer = uz > 0 ? 0 : S->L - 1;
    uint64_t events = 0;
    o->steps = 0;
    while (w > 0) {
        if (++events > 100000000ull) { w = 0; break; }
        double d;
        int next;
        if (uz < 0) { d = (S->bounds[layer] - z) / uz; next = layer - 1; }
        else if (uz > 0) { d = (S->bounds[layer + 1] - z) / uz; next = layer + 1; }
        else { d = INFINITY; next = layer; }
        if (S->mus[layer] == 0) {
            if (!(d < INFINITY)) { w = 0; break; }        /* a slide cannot be left */
            const double wn = w * exp(-S->mua[layer] * d);
            A += w - wn;
            w = wn;
        } else {
            const double s = tau / S->mut[layer];
            if (s < d) {
                /* hop, drop, roulette, spin, next free path (MLMC.py:165-200) */
                z += s * uz;
                ++o->steps;
                const double dW = w * S->mua[layer] / S->mut[layer];
                w -= dW;
                A += dW;
                if (w <= threshold) w = (uniform(g) <= 1.0 / m) ? m * w : 0;
                if (w > 0) {
                    ref_spin(S->g[layer], g, &ux, &uy, &uz);
                    double u = uniform(g);
                    if (u <= 0) u = 1e-300;
                    tau = -log(u);
                }
                continue;
            }
            tau -= d * S->mut[layer];
        }
        z = uz > 0 ? S->bounds[layer + 1] : S->bounds[layer];
        const double nn = (next == S->L || next == -1) ? 1.0 : S->n[next];
        if (uniform(g) < ref_fresnel_snell(S->n[layer], nn, uz)) {
            uz *= -1;
        } else {
            ref_snell(S->n[layer], nn, &ux, &uy, &uz);
            if (next == S->L) { Tr += w; w = 0; break; }
            if (next == -1) { Rf += w; w = 0; break; }
            layer = next;
        }
    }
    o->absorbed = A; o->reflected = Rf; o->transmitted = Tr; o->ux = ux; o->uy = uy; o->uz = uz;
}

typedef struct {
    int single;     /* 1: ISMC.py driver (one slab), 0: ISMLMC.py driver */
    int physical;   /* ISMC_MODE_PHYSICAL (stack driver only) */
    Stack S;
    ismc_spheres P;
    double threshold, m;
} Setup;

/* Sphere logic after a packet meets side 'r' (0) or 't' (1) with weight w:
 * returns 1 when the packet is re-incident (direction updated), else scores it.
 * ISMC.py:190-284 (incident reflection) and 298-399 (after the walk). */
static int ref_sphere(const Setup* st, int side, double w, double* ux, double* uy, double* uz,
                      Rng* g, double x[5]) {
    const ismc_spheres* P = &st->P;
    const int present = side ? P->T : P->R;
    if (present) {
        const double fp = side ? P->T_fp : P->R_fp;
        if (fabs(*uz) >= sqrt(1 - fp)) { x[side ? ISMC_T_TU : ISMC_T_RS] += w; return 0; }
        const double pw = side ? P->T_pw : P->R_pw, fs = side ? P->T_fs : P->R_fs,
                     f = side ? P->T_f : P->R_f;
        if (uniform(g) < (pw * fs) / (1 - pw * (1 - f))) {
            /* mu_z ~ U (ISMC.py:207); cosine-weighted sqrt(U) in physical mode */
            const double mz = st->physical ? sqrt(uniform(g)) : uniform(g);
            const double phi = 2 * M_PI * uniform(g);
            *uz = side ? -1 * mz : mz;
            *ux = cos(phi) * sqrt(1 - (*uz) * (*uz));
            *uy = sin(phi) * sqrt(1 - (*uz) * (*uz));
            return 1;
        }
        x[side ? ISMC_T_TD : ISMC_T_RD] += w;
        return 0;
    }
    const double ang = side ? P->T_angle : P->R_angle;
    const double fp = 0.5 * (1 - cos(2 * ang));
    if (fabs(*uz) >= sqrt(1 - fp)) x[side ? ISMC_T_TU : ISMC_T_RS] += w;
    else x[side ? ISMC_T_TD : ISMC_T_RD] += w;
    return 0;
}

static void ref_packet(const Setup* st, Rng* g, double x[5], uint64_t* steps) {
    const Stack* S = &st->S;
    double t_tot = 0;
    for (int l = 0; l < S->L; ++l) t_tot += S->t[l];
    double w = 1, z = 0, ux, uy, uz;
    if (st->P.specular_included) { ux = sqrt(1 - 0.99 * 0.99); uy = 0; uz = 0.99; }
    else { ux = 0; uy = 0; uz = 1; }
    int side = 0;
    for (int k = 0; k < 5; ++k) x[k] = 0;
    while (w > 0) {
        const int layer = uz > 0 ? 0 : S->L - 1;
        int reflect;
        if (st->single) {
            reflect = !(uniform(g) > ref_fresnel_snell(1.0, S->n[0], uz));
        } else if (st->physical) {
            /* one Fresnel draw at the outer face; a slide's inner face is
             * met by the walk */
            reflect = uniform(g) < ref_fresnel_snell(1.0, S->n[layer], uz);
        } else if (S->mus[layer] == 0.0) {
            const double n1 = 1.0, n2 = S->n[layer];
            const double n3 = uz > 0 ? (layer + 1 < S->L ? S->n[layer + 1] : 1.0)
                                     : (layer >= 1 ? S->n[layer - 1] : 1.0);
            const double r1 = ref_fresnel_snell(n1, n2, uz), r2 = ref_fresnel_snell(n2, n3, uz);
            reflect = uniform(g) < r1 + ((1 - r1) * (1 - r1)) * r2 / (1 - r1 * r2);
        } else {
            reflect = uniform(g) < ref_fresnel_snell(1.0, S->n[layer], uz);
        }
        if (reflect) {
            if (ref_sphere(st, side, w, &ux, &uy, &uz, g, x)) {
                z = side ? t_tot : 0;
                continue;
            }
            break;
        }
        ref_snell(1.0, S->n[layer], &ux, &uy, &uz);
        Walk o;
        if (st->single) {
            ref_mc_single(S, w, z, ux, uy, uz, g, &o);
        } else if (st->physical) {
            double u = uniform(g);
            if (u <= 0) u = 1e-300;
            ref_mc_multi_physical(S, w, z, ux, uy, uz, -log(u), g, st->threshold, st->m, &o);
        } else {
            ref_mc_multi(S, w, z, ux, uy, uz, g, st->threshold, st->m, &o);
        }
        *steps += o.steps;
        x[ISMC_T_A] += o.absorbed;
        ux = o.ux; uy = o.uy; uz = o.uz;
        if (o.reflected) { side = 0; w = o.reflected; }
        else if (o.transmitted) { side = 1; w = o.transmitted; }
        else break;
        if (ref_sphere(st, side, w, &ux, &uy, &uz, g, x)) {
            z = side ? t_tot : 0;
            continue;
        }
        break;
    }
}

typedef struct {
    const Setup* st;
    uint64_t seed, first, count;
    uint32_t stream;
    double sum[5], sumsq[5];
    uint64_t steps;
} Job;

static void* job_fn(void* arg) {
    Job* j = (Job*)arg;
    double x[5];
    for (uint64_t k = 0; k < j->count; ++k) {
        const uint64_t id = j->first + k;
        Rng g;
        memset(&g, 0, sizeof g);
        g.k0 = (uint32_t)j->seed; g.k1 = (uint32_t)(j->seed >> 32);
        g.c1 = (uint32_t)id; g.c2 = (uint32_t)(id >> 32); g.c3 = j->stream;
        g.idx = 4;
        ref_packet(j->st, &g, x, &j->steps);
        for (int i = 0; i < 5; ++i) { j->sum[i] += x[i]; j->sumsq[i] += x[i] * x[i]; }
    }
    return NULL;
}

/*
 * Run an instance through the restated reference.  single = 1 selects the
 * ISMC.py driver (single slab, roulette threshold from the instance, usually
 * 1e-3), 0 the ISMLMC.py driver.  sum/sumsq receive per-packet sums (FP64).
 */
int ref64_run(int single, const ismc_instance* inst, int threads, double sum[5], double sumsq[5],
              uint64_t* steps) {
    if (!inst || inst->stack.L < 1 || inst->stack.L > ISMC_MAXL) return -1;
    if (single && inst->stack.L != 1) return -1;
    Setup st;
    memset(&st, 0, sizeof st);
    st.single = single;
    st.physical = !single && inst->mode == ISMC_MODE_PHYSICAL;
    st.S.L = (int)inst->stack.L;
    st.S.bounds[0] = 0;
    for (int l = 0; l < st.S.L; ++l) {
        st.S.n[l] = inst->stack.n[l];
        st.S.mua[l] = inst->stack.mua[l];
        st.S.mus[l] = inst->stack.mus[l];
        st.S.mut[l] = inst->stack.mut[l];
        st.S.g[l] = inst->stack.g[l];
        st.S.t[l] = inst->stack.d[l];
        st.S.bounds[l + 1] = st.S.bounds[l] + st.S.t[l];
    }
    st.P = inst->spheres;
    st.threshold = inst->roulette_threshold;
    st.m = inst->roulette_m;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    Job jobs[256];
    pthread_t th[256];
    const uint64_t n = inst->n_packets;
    for (int k = 0; k < threads; ++k) {
        memset(&jobs[k], 0, sizeof(Job));
        jobs[k].st = &st;
        jobs[k].seed = inst->seed;
        jobs[k].stream = inst->stream;
        jobs[k].first = inst->packet_offset + n * (uint64_t)k / (uint64_t)threads;
        jobs[k].count = inst->packet_offset + n * (uint64_t)(k + 1) / (uint64_t)threads - jobs[k].first;
        pthread_create(&th[k], NULL, job_fn, &jobs[k]);
    }
    for (int i = 0; i < 5; ++i) { sum[i] = 0; sumsq[i] = 0; }
    *steps = 0;
    for (int k = 0; k < threads; ++k) {
        pthread_join(th[k], NULL);
        for (int i = 0; i < 5; ++i) { sum[i] += jobs[k].sum[i]; sumsq[i] += jobs[k].sumsq[i]; }
        *steps += jobs[k].steps;
    }
    return 0;
}
