// ismc_praxis.cpp -- PRAXIS (Brent 1973, ch. 7) as resumable coroutines.
// See ismc_praxis.h for the method summary.  Replaces the serial praxis()
// call of CUDA/ISMLMC-minimization.cu:476 (one blocking GPU launch per
// objective evaluation) with a form that a batch driver can interleave.
#include "ismc_praxis.h"

#include <cfloat>
#include <cmath>
#include <cstring>

namespace ismc {

static double urand(Praxis& s) {   // xorshift64*, uniform in [0,1)
    s.rng ^= s.rng >> 12;
    s.rng ^= s.rng << 25;
    s.rng ^= s.rng >> 27;
    return (double)((s.rng * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
}

static double norm(const double* a, int n) {
    double q = 0;
    for (int i = 0; i < n; ++i) q += a[i] * a[i];
    return std::sqrt(q);
}

// f at x + l v_j (j >= 0), or at the point of parameter l on the quadratic
// curve through q0 (l = -qd0), x (l = 0) and q1 (l = qd1) when j < 0.
static Task<double> flin(Praxis& s, int j, double l) {
    if (j >= 0) {
        for (int i = 0; i < s.n; ++i) s.point[i] = s.x[i] + l * s.v[i][j];
    } else {
        s.qa = l * (l - s.qd1) / (s.qd0 * (s.qd0 + s.qd1));
        s.qb = (l + s.qd0) * (s.qd1 - l) / (s.qd0 * s.qd1);
        s.qc = l * (l + s.qd0) / (s.qd1 * (s.qd0 + s.qd1));
        for (int i = 0; i < s.n; ++i) s.point[i] = s.qa * s.q0[i] + s.qb * s.x[i] + s.qc * s.q1[i];
    }
    ++s.nf;
    if (s.nf > s.maxfun) s.stopped = true;
    co_return co_await EvalAwait{&s};
}

// Safeguarded parabolic line search along direction j (or the curve, j < 0).
// d2: estimate of half the second derivative along the line (updated);
// x1: on entry an initial step (f1 its value when fk), on exit the step taken;
// at most nits extra halvings.
static Task<int> minline(Praxis& s, int j, int nits, double& d2, double& x1, double& f1,
                         bool fk) {
    const double sf1 = f1, sx1 = x1;
    int k = 0;
    double xm = 0, fm = s.fx;
    const double f0 = s.fx;
    bool dz = d2 < s.machep;
    double sn = norm(s.x, s.n);
    const double temp = dz ? s.dmin : d2;
    double t2 = s.m4 * std::sqrt(std::fabs(s.fx) / temp + sn * s.ldt) + s.m2 * s.ldt;
    sn = s.m4 * sn + s.t;
    if (dz && t2 > sn) t2 = sn;
    if (t2 < s.small) t2 = s.small;
    if (t2 > 0.01 * s.h) t2 = 0.01 * s.h;
    if (fk && f1 <= fm) { xm = x1; fm = f1; }
    if (!fk || std::fabs(x1) < t2) {
        x1 = x1 >= 0 ? t2 : -t2;
        f1 = co_await flin(s, j, x1);
    }
    if (f1 <= fm) { xm = x1; fm = f1; }
    double x2 = xm, f2 = fm;
    for (;;) {
        if (s.stopped) break;
        if (dz) {
            // one more point to estimate the curvature
            x2 = f0 < f1 ? -x1 : 2 * x1;
            f2 = co_await flin(s, j, x2);
            if (f2 <= fm) { xm = x2; fm = f2; }
            d2 = (x2 * (f1 - f0) - x1 * (f2 - f0)) / ((x1 - x2) * x1 * x2);
        }
        // minimum of the parabola through (0,f0), (x1,f1) with curvature d2
        const double d1 = (f1 - f0) / x1 - x1 * d2;
        dz = true;
        if (d2 <= s.small) x2 = d1 < 0 ? s.h : -s.h;
        else x2 = -0.5 * d1 / d2;
        if (std::fabs(x2) > s.h) x2 = x2 > 0 ? s.h : -s.h;
        bool again = false;
        for (;;) {
            f2 = co_await flin(s, j, x2);
            if (k < nits && f2 > f0 && !s.stopped) {
                ++k;
                if (f0 < f1 && x1 * x2 > 0) { again = true; break; }
                x2 *= 0.5;
                continue;
            }
            break;
        }
        if (!again) break;
    }
    ++s.nl;
    if (f2 > fm) x2 = xm; else fm = f2;
    if (std::fabs(x2 * (x2 - x1)) > s.small)
        d2 = (x2 * (f1 - f0) - x1 * (fm - f0)) / ((x1 - x2) * x1 * x2);
    else if (k > 0)
        d2 = 0;
    if (d2 <= s.small) d2 = s.small;
    x1 = x2;
    s.fx = fm;
    if (sf1 < s.fx) { s.fx = sf1; x1 = sx1; }
    if (j >= 0)
        for (int i = 0; i < s.n; ++i) s.x[i] += x1 * s.v[i][j];
    co_return 0;
}

// Quadratic extrapolation through the last three base points.
static Task<int> quad(Praxis& s) {
    double sv = s.fx;
    s.fx = s.qf1;
    s.qf1 = sv;
    s.qd1 = 0;
    for (int i = 0; i < s.n; ++i) {
        const double xi = s.x[i], l = s.q1[i];
        s.x[i] = l;
        s.q1[i] = xi;
        s.qd1 += (xi - l) * (xi - l);
    }
    s.qd1 = std::sqrt(s.qd1);
    double l = s.qd1, sc = 0;
    if (s.qd0 > 0 && s.qd1 > 0 && s.nl >= 3 * s.n * s.n) {
        double value = s.qf1;
        co_await minline(s, -1, 2, sc, l, value, true);
        s.qa = l * (l - s.qd1) / (s.qd0 * (s.qd0 + s.qd1));
        s.qb = (l + s.qd0) * (s.qd1 - l) / (s.qd0 * s.qd1);
        s.qc = l * (l + s.qd0) / (s.qd1 * (s.qd0 + s.qd1));
    } else {
        s.fx = s.qf1;
        s.qa = 0;
        s.qb = 0;
        s.qc = 1;
    }
    s.qd0 = s.qd1;
    for (int i = 0; i < s.n; ++i) {
        const double q = s.q0[i];
        s.q0[i] = s.x[i];
        s.x[i] = (s.qa * q + s.qb * s.x[i]) + s.qc * s.q1[i];
    }
    co_return 0;
}

// Left singular vectors and singular values of the n x n matrix m (columns =
// scaled directions) by one-sided Jacobi rotations on m^T.  On exit
// v[.][j] = j-th left singular vector, sv[j] = j-th singular value.
static void principal_axes(int n, double m[PRAXIS_NMAX][PRAXIS_NMAX],
                           double v[PRAXIS_NMAX][PRAXIS_NMAX], double* sv) {
    double a[PRAXIS_NMAX][PRAXIS_NMAX];   // a = m^T, columns rotated in place
    double w[PRAXIS_NMAX][PRAXIS_NMAX];   // accumulated rotations
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            a[i][j] = m[j][i];
            w[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double alpha = 0, beta = 0, gamma = 0;
                for (int i = 0; i < n; ++i) {
                    alpha += a[i][p] * a[i][p];
                    beta += a[i][q] * a[i][q];
                    gamma += a[i][p] * a[i][q];
                }
                if (gamma == 0) continue;
                off = std::fmax(off, std::fabs(gamma) / std::sqrt(alpha * beta));
                const double zeta = (beta - alpha) / (2 * gamma);
                const double tt = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
                const double c = 1 / std::sqrt(1 + tt * tt), sn = c * tt;
                for (int i = 0; i < n; ++i) {
                    const double ap = a[i][p], aq = a[i][q];
                    a[i][p] = c * ap - sn * aq;
                    a[i][q] = sn * ap + c * aq;
                    const double wp = w[i][p], wq = w[i][q];
                    w[i][p] = c * wp - sn * wq;
                    w[i][q] = sn * wp + c * wq;
                }
            }
        if (off < 1e-15) break;
    }
    for (int j = 0; j < n; ++j) {
        double q = 0;
        for (int i = 0; i < n; ++i) q += a[i][j] * a[i][j];
        sv[j] = std::sqrt(q);
        for (int i = 0; i < n; ++i) v[i][j] = w[i][j];
    }
}

Task<int> praxis_run(Praxis& s) {
    const int n = s.n;
    s.machep = DBL_EPSILON;
    s.small = s.machep * s.machep;
    s.vsmall = s.small * s.small;
    s.large = 1.0 / s.small;
    s.vlarge = 1.0 / s.vsmall;
    s.m2 = std::sqrt(s.machep);
    s.m4 = std::sqrt(s.m2);
    s.illc = false;
    double ldfac = 0.01;
    int kt = 0;
    s.nl = 0;
    s.nf = 1;
    for (int i = 0; i < n; ++i) s.point[i] = s.x[i];
    s.fx = co_await EvalAwait{&s};
    s.qf1 = s.fx;
    s.t = s.small + std::fabs(s.t0);
    double t2 = s.t;
    s.dmin = s.small;
    s.h = s.h0 < 100 * s.t ? 100 * s.t : s.h0;
    s.ldt = s.h;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) s.v[i][j] = i == j ? 1.0 : 0.0;
        s.d[i] = 0;
        s.q0[i] = s.x[i];
        s.q1[i] = s.x[i];
    }
    s.qd0 = 0;

    while (!s.stopped) {
        // ---- minimise along the first direction
        double sf = s.d[0];
        s.d[0] = 0;
        double step = 0, value = s.fx;
        co_await minline(s, 0, 2, s.d[0], step, value, false);
        if (step <= 0)
            for (int i = 0; i < n; ++i) s.v[i][0] = -s.v[i][0];
        if (sf <= 0.9 * s.d[0] || 0.9 * sf >= s.d[0])
            for (int i = 1; i < n; ++i) s.d[i] = 0;

        for (int k = 1; k < n && !s.stopped; ++k) {
            for (int i = 0; i < n; ++i) s.y[i] = s.x[i];
            sf = s.fx;
            if (kt > 0) s.illc = true;
            int kl = k;
            for (;;) {
                kl = k;
                double df = 0;
                if (s.illc) {
                    // random step off a possible resolution valley
                    for (int i = 0; i < n; ++i) {
                        const double r = (0.1 * s.ldt + t2 * std::pow(10.0, kt)) * (urand(s) - 0.5);
                        s.z[i] = r;
                        for (int j = 0; j < n; ++j) s.x[j] += r * s.v[j][i];
                    }
                    for (int i = 0; i < n; ++i) s.point[i] = s.x[i];
                    ++s.nf;
                    s.fx = co_await EvalAwait{&s};
                }
                // the non-conjugate directions k..n-1
                for (int k2 = k; k2 < n; ++k2) {
                    const double sl = s.fx;
                    double st = 0;
                    value = s.fx;
                    co_await minline(s, k2, 2, s.d[k2], st, value, false);
                    const double gain = s.illc ? s.d[k2] * (st + s.z[k2]) * (st + s.z[k2]) : sl - s.fx;
                    if (df <= gain) { df = gain; kl = k2; }
                }
                if (s.illc || df >= std::fabs(100 * s.machep * s.fx) || s.stopped) break;
                s.illc = true;
            }
            // the conjugate directions 0..k-1
            for (int k2 = 0; k2 < k && !s.stopped; ++k2) {
                double st = 0;
                value = s.fx;
                co_await minline(s, k2, 2, s.d[k2], st, value, false);
            }
            const double f1 = s.fx;
            s.fx = sf;
            double lds = 0;
            for (int i = 0; i < n; ++i) {
                double sl = s.x[i];
                s.x[i] = s.y[i];
                sl -= s.y[i];
                s.y[i] = sl;
                lds += sl * sl;
            }
            lds = std::sqrt(lds);
            if (lds > s.small) {
                // drop direction kl, make the net displacement direction k
                for (int i = kl - 1; i >= k; --i) {
                    for (int j = 0; j < n; ++j) s.v[j][i + 1] = s.v[j][i];
                    s.d[i + 1] = s.d[i];
                }
                s.d[k] = 0;
                for (int i = 0; i < n; ++i) s.v[i][k] = s.y[i] / lds;
                value = f1;
                co_await minline(s, k, 4, s.d[k], lds, value, true);
                if (lds <= 0) {
                    lds = -lds;
                    for (int i = 0; i < n; ++i) s.v[i][k] = -s.v[i][k];
                }
            }
            s.ldt *= ldfac;
            if (s.ldt < lds) s.ldt = lds;
            t2 = s.m2 * norm(s.x, n) + s.t;
            if (s.ldt > 0.5 * t2) kt = -1;
            ++kt;
            if (kt > s.ktm) { s.done = true; co_return 0; }
        }
        if (s.stopped) break;
        // ---- curved valley: extrapolate along the quadratic through the last points
        co_await quad(s);
        double dn = 0;
        for (int i = 0; i < n; ++i) {
            s.d[i] = 1.0 / std::sqrt(s.d[i]);
            if (dn < s.d[i]) dn = s.d[i];
        }
        double m[PRAXIS_NMAX][PRAXIS_NMAX];
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) m[i][j] = (s.d[j] / dn) * s.v[i][j];
        double sv[PRAXIS_NMAX];
        principal_axes(n, m, s.v, sv);
        for (int i = 0; i < n; ++i) {
            const double q = dn * sv[i];
            s.d[i] = q > s.large ? s.vsmall : (q < s.small ? s.vlarge : 1.0 / (q * q));
        }
        // sort by decreasing d (curvature estimate)
        for (int i = 0; i < n - 1; ++i) {
            int kbest = i;
            for (int j = i + 1; j < n; ++j)
                if (s.d[j] > s.d[kbest]) kbest = j;
            if (kbest != i) {
                std::swap(s.d[i], s.d[kbest]);
                for (int r = 0; r < n; ++r) std::swap(s.v[r][i], s.v[r][kbest]);
            }
        }
        s.dmin = s.d[n - 1] < s.small ? s.small : s.d[n - 1];
        s.illc = s.m4 * s.d[0] > s.dmin;
    }
    s.done = true;
    co_return 0;
}

double praxis_minimize(double (*f)(const double* x, int n, void* ctx), void* ctx, int n,
                       double* x, double t0, double h0, int maxfun, int* nf_out) {
    Praxis s;
    s.n = n;
    s.t0 = t0;
    s.h0 = h0;
    s.maxfun = maxfun;
    for (int i = 0; i < n; ++i) s.x[i] = x[i];
    Task<int> task = praxis_run(s);
    task.h.resume();
    while (!task.h.done()) {
        s.value = f(s.point, n, ctx);
        s.waiting.resume();
    }
    for (int i = 0; i < n; ++i) x[i] = s.x[i];
    if (nf_out) *nf_out = s.nf;
    return s.fx;
}

}  // namespace ismc
