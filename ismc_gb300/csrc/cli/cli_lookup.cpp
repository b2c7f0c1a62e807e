// Lookup.o -- drop-in for the reference's lookup-table data generator
// (CUDA/ISMLMC-lookup.cu), as Lookup/lookup.py:161-214 invokes it:
//
//   Lookup.o --GPU "0 1" (-N N --runs R | --unc U [--est E]) -n n -g g -t t
//            --Nmua A --muaS a0 --muaB ab --Nmus S --musS s0 --musB sb
//            [--Rangle deg] [--Tangle deg] [--Rsphere "pw fs fp fd"]
//            [--Tsphere "pw fs fp fd"] [--separate] [--specularIncluded] [--go]
//            [--seed K]
//
// Same flags, exit codes and output files: Diffuse_Reflectance.csv and
// Diffuse_Transmittance.csv in the working directory, each the grid of run
// averages followed by the grid of standard errors in the layout of
// write_data (ISMLMC-lookup.cu:112-150).  What differs is how the grid runs:
// every (run, mu_a, mu_s', sphere set) simulation of the whole table is one
// instance of a single batched launch per GPU (ismc_run_batch), instead of
// one launch per grid point.  The physics is the Python reference's
// (ISMLMC.py / MLMC.py, compat mode).  --seed is an addition (the reference
// seeds from the clock; so does this program without it).
#include <algorithm>
#include <fstream>
#include <iostream>
#include <thread>

#include "cli_common.h"

using cli::Args;

// write_data (ISMLMC-lookup.cu:112-150): header line, mu_s' line, one line per mu_a
static void write_data(const std::string& filename, const std::string& header, int N_mu_a,
                       int N_mu_s, const std::vector<float>& mu_a, const std::vector<float>& mu_s_,
                       const std::vector<float>& data, bool first) {
    std::ofstream file(filename, first ? std::ios::out : std::ios::app);
    file << "\"" << header << "\",\"mua\"";
    for (int i = 0; i < N_mu_s; ++i) file << ",\"\"";
    file << "\n";
    file << "\"mus'\",\"\"";
    for (int i = 0; i < N_mu_s; ++i) file << "," << mu_s_[i];
    file << "\n";
    for (int i = 0; i < N_mu_a; ++i) {
        file << "\"\"," << mu_a[i];
        for (int j = 0; j < N_mu_s; ++j) file << "," << data[(size_t)i * N_mu_s + j];
        file << "\n";
    }
}

static void usage() {
    std::cout << "\nLookup-table data generator (integrating-sphere Monte Carlo on the GPU).\n"
                 "\nFlags:\n"
                 "  --help, -h          this text\n"
                 "  --GPU \"ids\"         device ids (several ids split the table between them)\n"
                 "  -N N --runs R       packets per simulation and independent runs per point\n"
                 "  --unc U [--est E]   instead of -N/--runs: N = ceil(E / U^2), one run,\n"
                 "                      Poisson standard errors sqrt(x / N)\n"
                 "  -n, -g, -t          refractive index, anisotropy, thickness (cm) of the slab\n"
                 "  --Nmua, --muaS, --muaB   mu_a[i] = muaS * muaB^i, 0 <= i < Nmua (1/cm)\n"
                 "  --Nmus, --musS, --musB   mu_s'[j] = musS * musB^j (reduced scattering, 1/cm)\n"
                 "  --Rsphere \"pw fs fp fd\", --Tsphere \"pw fs fp fd\"   sphere parameters\n"
                 "  --Rangle deg, --Tangle deg   acceptance angles when a sphere is absent\n"
                 "  --separate          R_d and T_d from separate single-sphere runs\n"
                 "  --specularIncluded  8 degree incidence\n"
                 "  --example           the example configuration\n"
                 "  --go                do not ask for confirmation\n"
                 "  --seed K            Philox key (default: from the system entropy source)\n"
                 "\nWrites Diffuse_Reflectance.csv and Diffuse_Transmittance.csv.\n\n";
}

int main(int argc, char** argv) {
    Args a{argc, argv};
    if (a.has("--help") || a.has("-h")) {
        usage();
        return 1;
    }
    if (!a.has("--GPU")) {
        std::cout << "Must specify device IDs with the --GPU flag.\nUse --help to see available options.\n";
        return 2;
    }
    std::vector<int> gpus = a.ints("--GPU");
    if (gpus.empty()) {
        std::cout << "No device id given to --GPU.\n";
        return 2;
    }
    const bool go = a.has("--go");
    cli::Sphere R, T;
    bool specular_included = false;
    int N = -1, runs = -1;
    float estimate = 1.0f, uncertainty = 0.0f;
    bool separate = false;
    float n, g, t;
    int N_mu_a, N_mu_s;
    float mu_a_start, mu_a_base, mu_s__start, mu_s__base;

    if (a.has("--example")) {
        cli::example_spheres(R, T);
        N = 100000; runs = 10; separate = true;
        n = 1.4f; g = 0.5f; t = 0.135f;
        N_mu_a = 13; mu_a_start = 0.5f; mu_a_base = 1.2f;
        N_mu_s = 11; mu_s__start = 10.0f; mu_s__base = 1.2f;
    } else {
        if ((a.has("-N") != a.has("--runs")) && !a.has("--unc")) {
            std::cout << "-N and --runs must be used in conjuction, not by themselves.\n";
            return 2;
        }
        if ((a.has("-N") || a.has("--runs")) && (a.has("--unc") || a.has("--est"))) {
            std::cout << "-N and --runs cannot be used with --unc or --est\n";
            return 2;
        }
        cli::read_spheres(a, R, T, specular_included);
        if (a.has("-N") && a.has("--runs")) {
            N = a.i("-N");
            runs = a.i("--runs");
        } else if (a.has("--unc")) {
            runs = 0;
            if (a.has("--est")) estimate = a.f("--est");
            uncertainty = a.f("--unc");
            N = (int)std::ceil(estimate / (uncertainty * uncertainty));
        }
        separate = a.has("--separate");
        n = a.f("-n"); g = a.f("-g"); t = a.f("-t");
        N_mu_a = a.i("--Nmua"); mu_a_start = a.f("--muaS"); mu_a_base = a.f("--muaB");
        N_mu_s = a.i("--Nmus"); mu_s__start = a.f("--musS"); mu_s__base = a.f("--musB");
    }
    std::printf("\n-N %d\n--runs %d\n-n %f\n-g %f\n-t %f\n--Nmua %d\n--muaS %f\n--muaB %f\n--Nmus %d\n"
                "--musS %f\n--musB %f\n--Rsphere \"%f %f %f %f\"\n--Rangle %f\n--Tsphere \"%f %f %f %f\"\n"
                "--Tangle %f\n",
                N, runs, n, g, t, N_mu_a, mu_a_start, mu_a_base, N_mu_s, mu_s__start, mu_s__base, R.pw,
                R.fs, R.fp, R.fd, R.angle * 180 / M_PI, T.pw, T.fs, T.fp, T.fd, T.angle * 180 / M_PI);
    if (!go) {
        std::cout << "\nPress [enter] to start or Ctrl+C to cancel.\n";
        std::getchar();
    }
    if (N <= 0 || N_mu_a <= 0 || N_mu_s <= 0 || !(n > 0) || !(t > 0) || !(g > -1 && g <= 1)) {
        std::cout << "Missing or invalid parameters.  Use --help to see available options.\n";
        return 2;
    }
    const bool poisson = runs == 0;
    if (poisson) runs = 1;

    // grids as the reference computes them (float start * pow(float base, i))
    std::vector<float> mu_a(N_mu_a), mu_s_(N_mu_s), mu_s(N_mu_s);
    for (int i = 0; i < N_mu_a; ++i) mu_a[i] = mu_a_start * std::pow((double)mu_a_base, i);
    for (int j = 0; j < N_mu_s; ++j) {
        mu_s_[j] = mu_s__start * std::pow((double)mu_s__base, j);
        mu_s[j] = g == 1.0f ? mu_s_[j] : mu_s_[j] / (1 - g);
    }

    // one instance per (run, mu_a, mu_s', sphere set)
    const int kinds = separate ? 2 : 1;
    const uint64_t seed = a.seed();
    std::vector<ismc_instance> inst;
    inst.reserve((size_t)runs * N_mu_a * N_mu_s * kinds);
    for (int r = 0; r < runs; ++r)
        for (int i = 0; i < N_mu_a; ++i)
            for (int j = 0; j < N_mu_s; ++j)
                for (int k = 0; k < kinds; ++k) {
                    ismc_instance x{};
                    x.stack = cli::slab(n, mu_a[i], mu_s[j], g, t);
                    cli::Sphere r_ = R, t_ = T;
                    if (separate) {          // R sphere alone, then T sphere alone
                        r_.present = k == 0;
                        t_.present = k == 1;
                    }
                    x.spheres = cli::spheres(r_, t_, specular_included);
                    x.n_packets = (uint64_t)N;
                    x.seed = seed;
                    x.stream = (uint32_t)inst.size();
                    x.mode = ISMC_MODE_COMPAT;
                    x.roulette_threshold = 1e-4f;
                    x.roulette_m = 10.0f;
                    inst.push_back(x);
                }
    if (separate && !(R.present && T.present)) {
        std::cout << "--separate needs both --Rsphere and --Tsphere.\n";
        return 2;
    }

    // split the instances between the devices: one context and thread each
    std::vector<ismc_tally> out(inst.size());
    const size_t nd = std::min(gpus.size(), inst.size());
    std::vector<int> rc(nd, 0);
    std::vector<std::string> err(nd);
    std::vector<std::thread> th;
    for (size_t d = 0; d < nd; ++d) {
        th.emplace_back([&, d] {
            const size_t a0 = inst.size() * d / nd, a1 = inst.size() * (d + 1) / nd;
            ismc_ctx* ctx = nullptr;
            rc[d] = ismc_init(gpus[d], &ctx);
            if (rc[d]) { err[d] = cli::last_error(nullptr); return; }
            rc[d] = ismc_run_batch(ctx, inst.data() + a0, (uint32_t)(a1 - a0), nullptr,
                                   out.data() + a0);
            if (rc[d]) err[d] = cli::last_error(ctx);
            ismc_destroy(ctx);
        });
    }
    for (auto& x : th) x.join();
    for (size_t d = 0; d < nd; ++d)
        if (rc[d]) {
            std::fprintf(stderr, "GPU %d: error %d: %s\n", gpus[d], rc[d], err[d].c_str());
            return 3;
        }

    // per-run grids of R_d and T_d (R_d + R_s and T_d + T_u without spheres,
    // ISMLMC-lookup.cu:288-305), then averages and standard errors
    const size_t P = (size_t)N_mu_a * N_mu_s;
    std::vector<float> Rd((size_t)runs * P), Td((size_t)runs * P);
    for (int r = 0; r < runs; ++r)
        for (int i = 0; i < N_mu_a; ++i)
            for (int j = 0; j < N_mu_s; ++j) {
                const size_t p = (size_t)i * N_mu_s + j, q = ((size_t)r * P + p) * kinds;
                float rd, td;
                if (separate) {
                    rd = (float)cli::tally_mean(out[q], ISMC_T_RD);
                    td = (float)cli::tally_mean(out[q + 1], ISMC_T_TD);
                } else if (R.present || T.present) {
                    rd = (float)cli::tally_mean(out[q], ISMC_T_RD);
                    td = (float)cli::tally_mean(out[q], ISMC_T_TD);
                } else {
                    rd = (float)(cli::tally_mean(out[q], ISMC_T_RD) + cli::tally_mean(out[q], ISMC_T_RS));
                    td = (float)(cli::tally_mean(out[q], ISMC_T_TD) + cli::tally_mean(out[q], ISMC_T_TU));
                }
                Rd[(size_t)r * P + p] = rd;
                Td[(size_t)r * P + p] = td;
                std::printf("RUN: %2d of %2d | mua: %8.4f mus: %8.4f | R_d %1.6f T_d %1.6f\n", r + 1,
                            runs, mu_a[i], mu_s_[j], rd, td);
            }
    auto avg = [&](const std::vector<float>& v) {          // array_avg: sum of x / runs
        std::vector<float> m(P, 0.0f);
        for (int r = 0; r < runs; ++r)
            for (size_t p = 0; p < P; ++p) m[p] += v[(size_t)r * P + p] / runs;
        return m;
    };
    auto unc = [&](const std::vector<float>& v, const std::vector<float>& m) {
        std::vector<float> s(P, 0.0f);
        if (poisson) {                                      // array_poisson: sqrt(x / N)
            for (size_t p = 0; p < P; ++p) s[p] = std::sqrt(v[p] / N);
            return s;
        }
        for (int r = 0; r < runs; ++r)                      // array_stderr: population sd / sqrt(runs)
            for (size_t p = 0; p < P; ++p) s[p] += std::pow(v[(size_t)r * P + p] - m[p], 2);
        for (size_t p = 0; p < P; ++p) s[p] = std::sqrt(s[p] / runs) / std::sqrt((float)runs);
        return s;
    };
    const auto Rm = avg(Rd), Tm = avg(Td);
    const auto Ru = unc(Rd, Rm), Tu = unc(Td, Tm);
    write_data("Diffuse_Reflectance.csv", "Average Diffuse Reflectance", N_mu_a, N_mu_s, mu_a, mu_s_, Rm,
               true);
    write_data("Diffuse_Transmittance.csv", "Average Diffuse Transmittance", N_mu_a, N_mu_s, mu_a, mu_s_,
               Tm, true);
    write_data("Diffuse_Reflectance.csv", "Standard Error in Diffuse Reflectance", N_mu_a, N_mu_s, mu_a,
               mu_s_, Ru, false);
    write_data("Diffuse_Transmittance.csv", "Standard Error in Diffuse Transmittance", N_mu_a, N_mu_s,
               mu_a, mu_s_, Tu, false);
    return 0;
}
