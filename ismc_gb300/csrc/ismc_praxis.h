// ismc_praxis.h -- Brent's principal-axis minimiser (PRAXIS) as a resumable
// coroutine, so that many independent minimisations advance in lockstep and
// every round of objective evaluations can be served by one batched launch.
//
// Written from the published method: R. P. Brent, "Algorithms for
// Minimization without Derivatives" (Prentice-Hall, 1973), chapter 7 --
// line searches by safeguarded parabolic interpolation along the current
// directions, Powell's replacement of the least useful direction by the
// net displacement, random steps when the problem looks ill-conditioned,
// quadratic extrapolation along the curve through the last three points, and
// a new orthogonal set of principal directions from a singular value
// decomposition (here: one-sided Jacobi) of the scaled direction matrix.
#pragma once
#include <coroutine>
#include <cstdint>
#include <exception>
#include <utility>

namespace ismc {

// Coroutine returning T that can be awaited by another coroutine (symmetric
// transfer back to the awaiting coroutine when it finishes).
template <class T>
struct Task {
    struct promise_type {
        T value{};
        std::coroutine_handle<> cont;
        Task get_return_object() {
            return Task{std::coroutine_handle<promise_type>::from_promise(*this)};
        }
        std::suspend_always initial_suspend() noexcept { return {}; }
        struct Final {
            bool await_ready() noexcept { return false; }
            std::coroutine_handle<> await_suspend(std::coroutine_handle<promise_type> h) noexcept {
                auto c = h.promise().cont;
                return c ? c : std::noop_coroutine();
            }
            void await_resume() noexcept {}
        };
        Final final_suspend() noexcept { return {}; }
        void return_value(T v) { value = std::move(v); }
        void unhandled_exception() { std::terminate(); }
    };
    std::coroutine_handle<promise_type> h;
    explicit Task(std::coroutine_handle<promise_type> x) : h(x) {}
    Task(Task&& o) noexcept : h(std::exchange(o.h, {})) {}
    Task(const Task&) = delete;
    ~Task() { if (h) h.destroy(); }
    bool await_ready() { return false; }
    std::coroutine_handle<> await_suspend(std::coroutine_handle<> c) {
        h.promise().cont = c;
        return h;
    }
    T await_resume() { return h.promise().value; }
};

constexpr int PRAXIS_NMAX = 8;

// State of one minimisation.  The objective is requested through `point`;
// the driver evaluates it, stores the value in `value` and resumes `waiting`.
struct Praxis {
    // problem
    int n = 2;
    double t0 = 1e-5, h0 = 1.0;
    int maxfun = 2000;
    int ktm = 1;
    uint64_t rng = 0x9E3779B97F4A7C15ull;
    // result / state
    double x[PRAXIS_NMAX]{};
    double fx = 0;
    int nf = 0, nl = 0;
    bool done = false, stopped = false;
    // objective plumbing
    double point[PRAXIS_NMAX]{};
    double value = 0;
    bool pending = false;
    std::coroutine_handle<> waiting;

    // internal
    double v[PRAXIS_NMAX][PRAXIS_NMAX]{};   // v[i][j]: component i of direction j
    double d[PRAXIS_NMAX]{}, q0[PRAXIS_NMAX]{}, q1[PRAXIS_NMAX]{}, z[PRAXIS_NMAX]{},
        y[PRAXIS_NMAX]{};
    double qf1 = 0, qd0 = 0, qd1 = 0, qa = 0, qb = 0, qc = 0;
    double dmin = 0, ldt = 0, t = 0, h = 0, machep = 0, small = 0, vsmall = 0, large = 0,
           vlarge = 0, m2 = 0, m4 = 0;
    bool illc = false;
};

// Awaitable: request f(p) from the driver.
struct EvalAwait {
    Praxis* s;
    bool await_ready() const noexcept { return false; }
    void await_suspend(std::coroutine_handle<> c) noexcept {
        s->waiting = c;
        s->pending = true;
    }
    double await_resume() noexcept {
        s->pending = false;
        return s->value;
    }
};

// The minimisation coroutine: on completion s.x holds the minimiser and s.fx
// the objective there.
Task<int> praxis_run(Praxis& s);

// Blocking convenience wrapper over a host callback (used for tests and for
// objectives that need no batching).  Returns the objective at the minimum.
double praxis_minimize(double (*f)(const double* x, int n, void* ctx), void* ctx, int n,
                       double* x, double t0, double h0, int maxfun, int* nf_out);

}  // namespace ismc
