// ismc_solve.cpp -- batched plain-path inverse solver over the C ABI.
//
// Each solve is a PRAXIS coroutine (ismc_praxis.h).  The driver resumes every
// active solve until it asks for an objective value, turns all requests of the
// round into one batch of Monte Carlo instances (1-3 per request), runs them
// with ONE ismc_run_batch launch, scores the reference's cost and resumes.
// Reference: minimization.py:201-271 (cost, Powell minimise, accept box with
// retry), CUDA/ISMLMC-minimization.cu:89-131 (cost) and :466-488 (PRAXIS runs
// with reject-and-retry, which is unbounded there and bounded here).
//
// Refits (no counterpart in the reference).  PRAXIS ends a minimisation after
// two iterations whose steps stay below its tolerance.  On a Monte Carlo
// objective that can happen far from the minimum, once its line searches
// probe steps at which the objective is rough: on a slab between slides at
// 2e5 packets per objective, a few percent of 200 fits from one start ended
// inside the box with residuals of 3-12 % (most at the starting mu_s'), the
// rest near 0.02 %.  A minimisation that ends inside the box with a cost above
// kRefitNoise times the objective's own Monte Carlo standard error (from the
// tallies' sums of squares, at its lowest-cost evaluation) is probed: four
// evaluations, kProbeStep either side along each axis.  A residual that only
// measurement noise leaves (three measurements for two unknowns) does not
// fall there; a fit that stopped short does.  When a probe reaches kRefitGain
// of the end cost, the minimisation runs again from that probe on the same
// objective, up to max_refits times; a refit that ends higher keeps the point
// it started from.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/ismc.h"
#include "ismc_praxis.h"

using ismc::Praxis;
using ismc::Task;

namespace {

enum SimKind { SIM_BOTH = 0, SIM_R = 1, SIM_T = 2, SIM_NONE = 3 };

constexpr double kRefitNoise = 5.0;
constexpr double kProbeStep = 0.03;     // relative step of the probes around an end point
constexpr double kRefitGain = 0.9;      // a probe or refit must reach this fraction of the cost
constexpr double kInfCost = 1e30;       // outside the domain or not finite

// PRAXIS minimises the square of the reference's cost.  The cost is a
// Euclidean norm of residuals, a cone at its minimum; its square has the same
// minimiser and is locally quadratic, which is what PRAXIS's parabolic line
// searches and quadratic valley model assume (Brent 1973, ch. 7).  Every
// cost the solver reports is the reference's (the square root).
inline double praxis_value(double cost) { return cost < kInfCost ? cost * cost : kInfCost; }
inline double reported_cost(double v) { return v < kInfCost ? std::sqrt(v) : kInfCost; }

struct Solve {
    const ismc_solve_req* req = nullptr;
    Praxis px;
    std::unique_ptr<Task<int>> task;
    uint32_t evals = 0, restarts = 0, rounds = 0, refits = 0;
    bool finished = false;
    // lowest cost among the current minimisation's evaluations and the Monte
    // Carlo standard error of the cost there; the end point (PRAXIS
    // coordinates) and end cost of the minimisation a refit started from
    double best_cost = INFINITY, best_noise = 0, fit_cost = INFINITY;
    double fit_x[2] = {0, 0};
    // probes around an end point that may have stopped short: pending probe
    // 0..3 (-1: none), the end point and its cost, the point under
    // evaluation, and the lowest probe
    int probe = -1;
    double probe_c[2] = {0, 0}, probe_cost = 0, probe_pt[2] = {0, 0};
    double probe_best = INFINITY, probe_bx[2] = {0, 0};
    int32_t status = ISMC_OK;
    // instances of the pending request
    int first = -1, count = 0;
    SimKind kinds[3];
};

inline double to_param(const ismc_solve_req& r, double u) { return r.log_coords ? std::exp(u) : u; }
inline double from_param(const ismc_solve_req& r, double v) { return r.log_coords ? std::log(v) : v; }
// a point in PRAXIS coordinates inside the accepted box
inline bool in_box(const ismc_solve_req& r, const double* p) {
    const double a = to_param(r, p[0]), b = to_param(r, p[1]);
    return a >= r.lo[0] && a <= r.hi[0] && b >= r.lo[1] && b <= r.hi[1];
}

// A new minimisation of solve s: from the request's initial guess, or from
// the end point of the previous one (a refit, in PRAXIS coordinates).
void start(Solve& s, uint32_t index, uint32_t attempt, const double* from = nullptr) {
    const ismc_solve_req& r = *s.req;
    s.px = Praxis();
    s.best_cost = INFINITY;
    s.best_noise = 0;
    s.px.n = 2;
    s.px.t0 = r.t0;
    s.px.h0 = r.h0;
    s.px.maxfun = r.max_evals ? (int)r.max_evals : 2000;
    s.px.rng = 0x243F6A8885A308D3ull ^ ((uint64_t)index << 20) ^ attempt;
    s.px.x[0] = from ? from[0] : from_param(r, r.x0[0]);
    s.px.x[1] = from ? from[1] : from_param(r, r.x0[1]);
    s.task = std::make_unique<Task<int>>(ismc::praxis_run(s.px));
    s.task->h.resume();   // runs to the first objective request
}

// The objective's Monte Carlo instances for the point p of solve s.
int build_request(Solve& s, uint32_t index, const double* p, std::vector<ismc_instance>& out) {
    const ismc_solve_req& r = *s.req;
    const double mua = to_param(r, p[0]), musr = to_param(r, p[1]);
    s.first = (int)out.size();
    s.count = 0;
    if (!(mua > 0) || !(musr > 0) || !std::isfinite(mua) || !std::isfinite(musr)) return 0;
    // outside the accepted box the objective is infinite without simulating:
    // the reference rejects such answers afterwards (minimization.py:267), and
    // simulating there (e.g. mu_s' of 1e4 /cm: ~1e5 steps per packet) would
    // stall the whole batched round.  An initial guess outside the box (the
    // reference's own example starts at (5, 45) for a [1,3] x [20,40] box)
    // widens the evaluated region on that side to take it in, with margin,
    // so that the search can walk from the guess into the box.
    const double elo0 = r.x0[0] < r.lo[0] ? r.x0[0] / 1.5 : r.lo[0];
    const double ehi0 = r.x0[0] > r.hi[0] ? r.x0[0] * 1.5 : r.hi[0];
    const double elo1 = r.x0[1] < r.lo[1] ? r.x0[1] / 1.5 : r.lo[1];
    const double ehi1 = r.x0[1] > r.hi[1] ? r.x0[1] * 1.5 : r.hi[1];
    if (mua < elo0 || mua > ehi0 || musr < elo1 || musr > ehi1) return 0;
    ismc_instance base = r.base;
    const uint32_t l = r.layer;
    const double g = base.stack.g[l];
    const double mus = g == 1.0 ? musr : musr / (1.0 - g);     // minimization.py:204-205
    base.stack.mua[l] = (float)mua;
    base.stack.mus[l] = (float)mus;
    base.stack.mut[l] = (float)(mua + mus);
    // independent Philox stream per (solve, evaluation, run kind)
    const uint32_t ev = s.evals;
    auto push = [&](SimKind k, bool R, bool T) {
        ismc_instance x = base;
        x.spheres.R = R ? 1 : 0;
        x.spheres.T = T ? 1 : 0;
        const uint32_t evk = r.fresh_streams ? ev : 0u;
        x.stream = (uint32_t)(index * 2654435761u) ^ (evk << 2) ^ (uint32_t)k;
        x.seed = r.base.seed + ((uint64_t)s.restarts << 40);
        out.push_back(x);
        s.kinds[s.count++] = k;
    };
    const bool hasRd = !std::isnan(r.meas[0]), hasRs = !std::isnan(r.meas[1]),
               hasTd = !std::isnan(r.meas[2]), hasTu = !std::isnan(r.meas[3]);
    if (r.separate) {
        if (hasRd) push(SIM_R, true, false);
        if (hasTd) push(SIM_T, false, true);
        if (hasRs || hasTu) push(SIM_NONE, false, false);
    } else {
        push(SIM_BOTH, base.spheres.R != 0, base.spheres.T != 0);
    }
    return s.count;
}

double tally_mean(const ismc_tally& t, int k) {
    return t.n ? (double)t.sum[k] / std::ldexp((double)t.n, (int)t.scale_log2) : NAN;
}

// variance of a tally's mean, (E[w^2] - E[w]^2) / (N - 1)
double tally_var(const ismc_tally& t, int k) {
    if (t.n < 2) return 0;
    const double n = (double)t.n, m = tally_mean(t, k);
    const double ex2 = (double)t.sumsq[k] / std::ldexp(n, (int)t.scale_log2);
    return std::max(ex2 - m * m, 0.0) / (n - 1);
}

// minimization.py:231-238; *noise = the cost's Monte Carlo standard error,
// sqrt of the sum of the terms' variances (relative terms scaled alike)
double score(const Solve& s, const ismc_tally* t, double* noise) {
    const ismc_solve_req& r = *s.req;
    double v[4] = {NAN, NAN, NAN, NAN}, var[4] = {0, 0, 0, 0};
    auto take = [&](int slot, const ismc_tally& x, int k) {
        v[slot] = tally_mean(x, k);
        var[slot] = tally_var(x, k);
    };
    for (int i = 0; i < s.count; ++i) {
        const ismc_tally& x = t[s.first + i];
        switch (s.kinds[i]) {
            case SIM_BOTH: take(0, x, ISMC_T_RD); take(1, x, ISMC_T_RS);
                           take(2, x, ISMC_T_TD); take(3, x, ISMC_T_TU); break;
            case SIM_R: take(0, x, ISMC_T_RD); break;
            case SIM_T: take(2, x, ISMC_T_TD); break;
            case SIM_NONE: take(1, x, ISMC_T_RS); take(3, x, ISMC_T_TU); break;
        }
    }
    double c = 0, nv = 0;
    for (int k = 0; k < 4; ++k) {
        if (std::isnan(r.meas[k])) continue;
        // R_d and T_d enter relative to the measurement, R_s and T_u absolute
        const double scale = (k == 0 || k == 2) ? 1.0 / r.meas[k] : 1.0;
        c += std::pow((v[k] - r.meas[k]) * scale, 2);
        nv += var[k] * scale * scale;
    }
    *noise = std::sqrt(nv);
    return std::isfinite(c) ? std::sqrt(c) : kInfCost;
}

// The answer of solve s: end point p (PRAXIS coordinates) and its cost.
void finish(Solve& s, ismc_solve_out& o, const double* p, double cost, bool inside) {
    const ismc_solve_req& r = *s.req;
    s.finished = true;
    s.status = inside ? ISMC_OK : ISMC_ERR_CAPACITY;
    o.x[0] = to_param(r, p[0]);
    o.x[1] = to_param(r, p[1]);
    o.cost = cost;
}

}  // namespace

extern "C" int ismc_praxis(ismc_objective f, void* user, int n, double* x, double t0, double h0,
                           int maxfun, double* fmin, int* nevals) {
    if (!f || !x || n < 1 || n > ismc::PRAXIS_NMAX || !(h0 > 0)) return ISMC_ERR_INVALID_ARG;
    double v = ismc::praxis_minimize(f, user, n, x, t0, h0, maxfun > 0 ? maxfun : 2000, nevals);
    if (fmin) *fmin = v;
    return ISMC_OK;
}

extern "C" int ismc_solve_batch(ismc_ctx* ctx, const ismc_solve_req* req, uint32_t n,
                                ismc_solve_out* out) {
    if (!ctx || !req || !out || n == 0) return ISMC_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i) {
        const ismc_solve_req& r = req[i];
        if (r.layer >= r.base.stack.L || r.base.stack.L > ISMC_MAXL || !(r.h0 > 0) ||
            !(r.x0[0] > 0) || !(r.x0[1] > 0) || r.base.n_packets == 0)
            return ISMC_ERR_INVALID_ARG;
    }
    std::vector<Solve> S(n);
    for (uint32_t i = 0; i < n; ++i) {
        S[i].req = &req[i];
        start(S[i], i, 0);
    }
    std::vector<ismc_instance> batch;
    std::vector<ismc_tally> tallies;
    std::vector<uint32_t> active;
    for (;;) {
        batch.clear();
        active.clear();
        for (uint32_t i = 0; i < n; ++i) {
            Solve& s = S[i];
            for (;;) {
                if (s.probe >= 4) {
                    // all probes in: refit from the lowest when it is clearly
                    // lower than the end point, else accept the end point
                    const double* c = s.probe_c;
                    if (s.probe_best < kRefitGain * s.probe_cost) {
                        s.fit_cost = s.probe_cost;
                        s.fit_x[0] = c[0];
                        s.fit_x[1] = c[1];
                        ++s.refits;
                        s.probe = -1;
                        start(s, i, s.restarts | (s.refits << 8), s.probe_bx);
                        continue;
                    }
                    s.probe = -1;
                    finish(s, out[i], c, s.probe_cost, true);
                    continue;
                }
                if (s.probe >= 0) {
                    // probe k: +-kProbeStep along axis k/2 of the end point
                    const ismc_solve_req& r = *s.req;
                    const int ax = s.probe >> 1;
                    const double sg = (s.probe & 1) ? -1.0 : 1.0;
                    s.probe_pt[0] = s.probe_c[0];
                    s.probe_pt[1] = s.probe_c[1];
                    s.probe_pt[ax] = r.log_coords ? s.probe_c[ax] + sg * kProbeStep
                                                  : s.probe_c[ax] * (1.0 + sg * kProbeStep);
                    if (!in_box(r, s.probe_pt) || build_request(s, i, s.probe_pt, batch) == 0) {
                        ++s.probe;          // a probe outside the box counts as no gain
                        continue;
                    }
                    active.push_back(i);
                    break;
                }
                if (!s.finished && s.task->h.done()) {
                    // a minimisation ended: probe it when it stopped short, accept,
                    // or restart when outside the box
                    const ismc_solve_req& r = *s.req;
                    double ex[2] = {s.px.x[0], s.px.x[1]};
                    double end_cost = reported_cost(s.px.fx);
                    bool inside = in_box(r, ex);
                    if (s.refits > 0 && (!inside || !(end_cost < s.fit_cost))) {
                        // a refit that found nothing lower (or left the box) keeps
                        // the end point it started from
                        ex[0] = s.fit_x[0];
                        ex[1] = s.fit_x[1];
                        end_cost = s.fit_cost;
                        inside = true;
                    }
                    if (inside && !s.px.stopped && s.refits < r.max_refits &&
                        end_cost > kRefitNoise * s.best_noise &&
                        end_cost < kRefitGain * s.fit_cost) {
                        s.probe = 0;
                        s.probe_c[0] = ex[0];
                        s.probe_c[1] = ex[1];
                        s.probe_cost = end_cost;
                        s.probe_best = INFINITY;
                        continue;
                    }
                    if (inside || s.restarts >= r.max_restarts) {
                        finish(s, out[i], ex, end_cost, inside);
                    } else {
                        ++s.restarts;
                        start(s, i, s.restarts);
                    }
                    continue;
                }
                if (s.finished) break;
                if (build_request(s, i, s.px.point, batch) == 0) {
                    // outside the physical domain: infinite cost, no simulation
                    s.px.value = kInfCost;
                    ++s.evals;
                    s.px.waiting.resume();
                    continue;
                }
                active.push_back(i);
                break;
            }
        }
        if (active.empty()) break;
        tallies.resize(batch.size());
        const int rc = ismc_run_batch(ctx, batch.data(), (uint32_t)batch.size(), nullptr,
                                      tallies.data());
        if (rc) return rc;
        for (uint32_t i : active) {
            Solve& s = S[i];
            double noise = 0;
            const double c = score(s, tallies.data(), &noise);
            ++s.evals;
            ++s.rounds;
            if (s.probe >= 0) {
                if (c < s.probe_best) {
                    s.probe_best = c;
                    s.probe_bx[0] = s.probe_pt[0];
                    s.probe_bx[1] = s.probe_pt[1];
                }
                ++s.probe;
                continue;
            }
            s.px.value = praxis_value(c);
            if (c < s.best_cost) {
                s.best_cost = c;
                s.best_noise = noise;
            }
            s.px.waiting.resume();
        }
    }
    for (uint32_t i = 0; i < n; ++i) {
        out[i].evals = S[i].evals;
        out[i].restarts = S[i].restarts;
        out[i].status = S[i].status;
        out[i].rounds = S[i].rounds;
        out[i].refits = S[i].refits;
    }
    return ISMC_OK;
}
