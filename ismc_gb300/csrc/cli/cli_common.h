// Command-line handling shared by the two drop-in programs (Lookup.o and
// minimize.o).  Option semantics follow the reference's CUDA/cmdlineparse.h:
//   - an option is present when any argv element equals it exactly;
//   - its value is the next argv element;
//   - a missing float option reads as NaN, a missing int option as -1;
//   - an array option is one argv element holding whitespace-separated floats
//     (the drivers quote them: --Rsphere "pw fs fp fd").
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "ismc.h"

namespace cli {

struct Args {
    int argc;
    char** argv;

    int find(const char* opt) const {
        for (int i = 1; i < argc; ++i)
            if (std::strcmp(argv[i], opt) == 0) return i;
        return -1;
    }
    bool has(const char* opt) const { return find(opt) >= 0; }
    const char* value(const char* opt) const {
        const int i = find(opt);
        return (i >= 0 && i + 1 < argc) ? argv[i + 1] : nullptr;
    }
    // float option -> NaN when absent (cmdlineparse.h:33-46: atof of the value)
    float f(const char* opt) const {
        const char* v = value(opt);
        return v ? (float)std::atof(v) : std::nanf("0");
    }
    // int option -> -1 when absent (cmdlineparse.h readIntOption)
    int i(const char* opt) const {
        const char* v = value(opt);
        return v ? std::atoi(v) : -1;
    }
    // whitespace-separated floats of one argument, NaN-padded to len
    std::vector<float> arr(const char* opt, int len) const {
        std::vector<float> out(len, std::nanf("1"));
        const char* v = value(opt);
        if (!v) return out;
        std::stringstream ss(v);
        float t;
        for (int k = 0; k < len && (ss >> t); ++k) out[k] = t;
        return out;
    }
    std::vector<int> ints(const char* opt) const {
        std::vector<int> out;
        const char* v = value(opt);
        if (!v) return out;
        std::stringstream ss(v);
        int t;
        while (ss >> t) out.push_back(t);
        return out;
    }
    // --seed S (an addition: the reference seeds from the clock)
    uint64_t seed() const {
        const char* v = value("--seed");
        if (v) return std::strtoull(v, nullptr, 10);
        std::random_device rd;
        return ((uint64_t)rd() << 32) ^ rd();
    }
};

// The sample as the reference's programs simulate it: one slab, no slides,
// ambient index 1 on both sides (ISMLMC-lookup.cu:719-729: layers = 1).
inline ismc_stack slab(float n, float mua, float mus, float g, float t) {
    ismc_stack s{};
    s.L = 1;
    s.n[0] = n;
    s.mua[0] = mua;
    s.mus[0] = mus;
    s.mut[0] = mua + mus;
    s.g[0] = g;
    s.d[0] = t;
    return s;
}

struct Sphere {
    bool present = false;
    float pw = std::nanf("0"), fs = std::nanf("0"), fp = std::nanf("0"), fd = std::nanf("0");
    float angle = 0.0f;   // radians
};

inline ismc_spheres spheres(const Sphere& R, const Sphere& T, bool specular_included) {
    ismc_spheres s{};
    s.R = R.present;
    s.T = T.present;
    s.specular_included = specular_included;
    s.R_pw = R.pw; s.R_fs = R.fs; s.R_fp = R.fp; s.R_fd = R.fd;
    s.R_f = (double)(R.fs + R.fp + R.fd);
    s.R_angle = R.angle;
    s.T_pw = T.pw; s.T_fs = T.fs; s.T_fp = T.fp; s.T_fd = T.fd;
    s.T_f = (double)(T.fs + T.fp + T.fd);
    s.T_angle = T.angle;
    // an absent sphere's parameters are unused; keep them finite for validation
    if (!s.R) { s.R_pw = s.R_fs = s.R_fp = s.R_fd = s.R_f = 0.0; }
    if (!s.T) { s.T_pw = s.T_fs = s.T_fp = s.T_fd = s.T_f = 0.0; }
    return s;
}

// --Rsphere "pw fs fp fd" / --Rangle deg, and the same for T (ISMLMC-lookup.cu:616-658)
inline void read_spheres(const Args& a, Sphere& R, Sphere& T, bool& specular_included) {
    R.present = a.has("--Rsphere");
    if (R.present) {
        auto p = a.arr("--Rsphere", 4);
        R.pw = p[0]; R.fs = p[1]; R.fp = p[2]; R.fd = p[3];
    }
    R.angle = a.has("--Rangle") ? (float)(a.f("--Rangle") * M_PI / 180) : 0.0f;
    specular_included = a.has("--specularIncluded");
    T.present = a.has("--Tsphere");
    if (T.present) {
        auto p = a.arr("--Tsphere", 4);
        T.pw = p[0]; T.fs = p[1]; T.fp = p[2]; T.fd = p[3];
    }
    T.angle = a.has("--Tangle") ? (float)(a.f("--Tangle") * M_PI / 180) : 0.0f;
}

// the example spheres of both programs (Cook et al. 2019 configuration)
inline void example_spheres(Sphere& R, Sphere& T) {
    R.present = true; R.pw = 0.99f; R.fs = 0.023510f; R.fp = 0.054638f; R.fd = 0.023510f;
    R.angle = 0.0f;
    T.present = true; T.pw = 0.99f; T.fs = 0.054638f; T.fp = 0.023510f; T.fd = 0.023510f;
    T.angle = (float)(0.22 * M_PI / 180);
}

inline double tally_mean(const ismc_tally& t, int k) {
    return t.n ? std::ldexp((double)t.sum[k], -(int)t.scale_log2) / (double)t.n : 0.0;
}

inline std::string last_error(ismc_ctx* ctx) {
    char buf[512];
    ismc_last_error(ctx, buf, sizeof buf);
    return buf;
}

}  // namespace cli
