// minimize.o -- drop-in for the reference's minimization solver
// (CUDA/ISMLMC-minimization.cu), as Minimization/minimization.py:169-196
// invokes it:
//
//   minimize.o --GPU id -N N --runs R --step h --tol t -n n -g g -t d
//              --Rangle deg --Tangle deg --Rsphere "pw fs fp fd" --Tsphere "pw fs fp fd"
//              --mua a0 --mus s0 --muaMin .. --muaMax .. --musMin .. --musMax ..
//              [--Rd x] [--Rs x] [--Td x] [--Tu x] [--separate] [--specularIncluded]
//              [--verbose] [--go] [--seed K] [--crn] [--maxEvals M]
//
// Same flags and the same stdout protocol: without --verbose it prints exactly
// four numbers, mean mu_a, its standard error, mean mu_s', its standard error
// (ISMLMC-minimization.cu:516), which minimization.py:186-196 parses.  Each of
// the R runs is a PRAXIS minimisation (step h, tolerance t) of the reference's
// cost (ISMLMC-minimization.cu:89-131) over (mu_a, mu_s') of the slab, each
// objective an N-packet Monte Carlo run.  What differs: all R runs advance in
// lockstep through ismc_solve_batch, one batched launch per round of
// objective evaluations; the cost is not simulated (infinite) outside the box
// [muaMin, muaMax] x [musMin, musMax], widened to take in an initial guess
// outside it; and a run that still ends outside the box is repeated at most
// 20 times instead of without limit.  By default every evaluation draws fresh random
// numbers, as the reference's global generator does; --crn makes each run reuse
// one Philox stream (common random numbers: a deterministic objective).
#include <iostream>

#include "cli_common.h"

using cli::Args;

int main(int argc, char** argv) {
    Args a{argc, argv};
    if (a.has("--help") || a.has("-h")) {
        std::cout << "\nMinimization solver for optical properties (integrating-sphere Monte Carlo on "
                     "the GPU).\n\nFlags: --GPU id, -N packets per objective, --runs R, --step h, --tol t,\n"
                     "-n, -g, -t (slab), --mua, --mus (start), --muaMin/--muaMax/--musMin/--musMax (box),\n"
                     "--Rd/--Rs/--Td/--Tu (measurements), --Rsphere/--Tsphere \"pw fs fp fd\",\n"
                     "--Rangle/--Tangle deg, --separate, --specularIncluded, --verbose, --go, --example,\n"
                     "--seed K, --crn (common random numbers), --maxEvals M (per run, default 2000).\n"
                     "Prints mua, its standard error, mus', its standard error.\n\n";
        return 1;
    }
    if (!a.has("--GPU")) {
        std::cout << "Must specify device ID with the --GPU flag.\nUse --help to see available options.\n";
        return 2;
    }
    const int GPU = a.i("--GPU");
    const bool go = a.has("--go");
    cli::Sphere R, T;
    bool specular_included = false, separate = false, verbose = false;
    int N, runs;
    double step, tolerance;
    float n, g, t, mua0, mus0, mua_min, mua_max, mus_min, mus_max;
    float Rd, Rs, Td, Tu;
    if (a.has("--example")) {
        cli::example_spheres(R, T);
        N = 10000; runs = 5; step = 5; separate = true; verbose = true;
        n = 1.4f; g = 0.5f; t = 0.135f;
        mua0 = 5; mus0 = 35;
        mua_min = 1; mua_max = 3; mus_min = 20; mus_max = 40;
        tolerance = 1;
        Rd = 0.2716f; Td = 0.0853f; Tu = 0.0f; Rs = std::nanf("0");
    } else {
        cli::read_spheres(a, R, T, specular_included);
        N = a.i("-N");
        runs = a.i("--runs");
        step = a.f("--step");
        separate = a.has("--separate");
        verbose = a.has("--verbose");
        n = a.arr("-n", 1)[0];
        g = a.arr("-g", 1)[0];
        t = a.arr("-t", 1)[0];
        Rd = a.f("--Rd"); Rs = a.f("--Rs"); Td = a.f("--Td"); Tu = a.f("--Tu");
        mua0 = a.arr("--mua", 1)[0];
        mus0 = a.arr("--mus", 1)[0];
        mua_min = a.f("--muaMin"); mua_max = a.f("--muaMax");
        mus_min = a.f("--musMin"); mus_max = a.f("--musMax");
        tolerance = a.f("--tol");
    }
    if (!go) {
        std::printf("\nParameters:\n\n-N %d\n--runs %d\n--step %f\n-n %f\n-g %f\n-t %f\n--mua %f\n--mus %f"
                    "\n--muaMin %f\n--muaMax %f\n--musMin %f\n--musMax %f\n--tol %f"
                    "\n--Rsphere \"%f %f %f %f\"\n--Rangle %f\n--Tsphere \"%f %f %f %f\"\n--Tangle %f"
                    "\n--Rd %f\n--Rs %f\n--Td %f\n--Tu %f\n",
                    N, runs, step, n, g, t, mua0, mus0, mua_min, mua_max, mus_min, mus_max, tolerance,
                    R.pw, R.fs, R.fp, R.fd, R.angle * 180 / M_PI, T.pw, T.fs, T.fp, T.fd,
                    T.angle * 180 / M_PI, Rd, Rs, Td, Tu);
        std::getchar();
    }
    if (N <= 0 || runs <= 0 || !(step > 0) || !(tolerance > 0) || !(n > 0) || !(t > 0) ||
        !(mua_min <= mua_max) || !(mus_min <= mus_max)) {
        std::cout << "Missing or invalid parameters.  Use --help to see available options.\n";
        return 2;
    }
    const uint64_t seed = a.seed();
    const bool crn = a.has("--crn");
    const int max_evals = a.has("--maxEvals") ? a.i("--maxEvals") : 2000;

    // mu_s = mu_s' / (1 - g) unless g == 1 (ISMLMC-minimization.cu:97-99): the
    // solver works on mu_s' of layer 0 and keeps its g
    std::vector<ismc_solve_req> req(runs);
    for (int r = 0; r < runs; ++r) {
        ismc_solve_req& q = req[r];
        q = ismc_solve_req{};
        q.base.stack = cli::slab(n, mua0, g == 1.0f ? mus0 : mus0 / (1 - g), g, t);
        q.base.spheres = cli::spheres(R, T, specular_included);
        q.base.n_packets = (uint64_t)N;
        q.base.seed = seed;
        q.base.stream = (uint32_t)r;
        q.base.mode = ISMC_MODE_COMPAT;
        q.base.roulette_threshold = 1e-4f;
        q.base.roulette_m = 10.0f;
        q.layer = 0;
        q.separate = separate ? 1 : 0;
        q.log_coords = 0;
        q.max_evals = (uint32_t)max_evals;
        q.max_restarts = 20;         // the reference repeats until inside, unbounded
        q.max_refits = 2;
        q.fresh_streams = crn ? 0 : 1;
        q.meas[0] = Rd; q.meas[1] = Rs; q.meas[2] = Td; q.meas[3] = Tu;
        q.x0[0] = mua0; q.x0[1] = mus0;
        q.lo[0] = mua_min; q.lo[1] = mus_min;
        q.hi[0] = mua_max; q.hi[1] = mus_max;
        q.h0 = step;
        q.t0 = tolerance;
    }
    ismc_ctx* ctx = nullptr;
    int rc = ismc_init(GPU, &ctx);
    if (rc) {
        std::fprintf(stderr, "GPU %d: error %d: %s\n", GPU, rc, cli::last_error(nullptr).c_str());
        return 3;
    }
    std::vector<ismc_solve_out> out(runs);
    rc = ismc_solve_batch(ctx, req.data(), (uint32_t)runs, out.data());
    if (rc) {
        std::fprintf(stderr, "GPU %d: error %d: %s\n", GPU, rc, cli::last_error(ctx).c_str());
        ismc_destroy(ctx);
        return 3;
    }
    ismc_destroy(ctx);
    int outside = 0;
    for (int r = 0; r < runs; ++r) outside += out[r].status != ISMC_OK;
    if (outside)
        std::fprintf(stderr, "warning: %d of %d runs ended outside the accepted box after %u restarts\n",
                     outside, runs, req[0].max_restarts);

    // mean and population standard deviation / sqrt(runs) (ISMLMC-minimization.cu:490-511)
    const float Nruns = (float)runs;
    double ma = 0, ms = 0;
    for (int r = 0; r < runs; ++r) {
        if (verbose)
            std::printf("RUN %d of %d: mua %f mus' %f cost %g evaluations %u\n", r + 1, runs, out[r].x[0],
                        out[r].x[1], out[r].cost, out[r].evals);
        ma += (1 / Nruns) * out[r].x[0];
        ms += (1 / Nruns) * out[r].x[1];
    }
    double sa = 0, ss = 0;
    for (int r = 0; r < runs; ++r) {
        sa += std::pow(out[r].x[0] - ma, 2);
        ss += std::pow(out[r].x[1] - ms, 2);
    }
    const double ea = std::sqrt((1 / Nruns) * sa) / std::sqrt(Nruns);
    const double es = std::sqrt((1 / Nruns) * ss) / std::sqrt(Nruns);
    if (verbose)
        std::printf("\n\nMinimization Finished. Recovered Optical Properties:\n\nmua: %f +/- %f\nmus': %f +/- %f\n\n",
                    ma, ea, ms, es);
    else
        std::printf("%f\n%f\n%f\n%f\n", ma, ea, ms, es);
    return 0;
}
