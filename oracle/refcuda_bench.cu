// refcuda_bench.cu -- timing harness for the reference's own CUDA forward model.
//
// Baseline infrastructure, not product code: it is compiled only by
// oracle/build_ref.py:build_refcuda(), against an unmodified staged copy of the
// reference's CUDA/CUDAISMLMC.h, and run only by bench.py's reference arm.
//
// It drives the reference's code two ways, on one layer stack:
//   e2e     the reference's host entry point ISMLMC() (CUDAISMLMC.h:656-755:
//           cudaSetDevice, per-call cudaMalloc/cudaMemcpy of every array,
//           kernel, cudaDeviceSynchronize, copies back, cudaFree), host clock;
//   kernel  the reference's kernel CUDAISMLMC (CUDAISMLMC.h:316-654) alone, with
//           the launch shape ISMLMC() uses (256 threads, N/256 + 1 blocks) on
//           device-resident arrays, CUDA events on the launching stream.
// Each call simulates N packets.  The reference keeps one curand state per
// thread in an array of RNGS states that its first ISMLMC() call on a device
// initialises for that call's grid only (CUDAISMLMC.h:12, 662-683); every call
// here therefore has the same N, N + 256 <= RNGS, and the first call is an
// untimed ISMLMC() warm-up.
//
// Usage: refcuda_bench --layers L -n "n0 n1 .." -g ".." -t ".." --mua ".." --mus ".."
//            [--Rsphere "pw fs fp fd"] [--Tsphere "pw fs fp fd"] [--Rangle deg] [--Tangle deg]
//            --packets N --calls K
// --mus is the scattering coefficient mu_s itself (ISMLMC() takes mu_s and
// mu_t = mu_a + mu_s).  Prints one JSON line.
#include "CUDAISMLMC.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

const char* opt(int argc, char** argv, const char* name) {
    for (int i = 1; i + 1 < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return argv[i + 1];
    return nullptr;
}

std::vector<float> floats(const char* s, size_t want, const char* name) {
    std::vector<float> v;
    if (s) {
        char* end = nullptr;
        const char* p = s;
        for (;;) {
            const float x = std::strtof(p, &end);
            if (end == p) break;
            v.push_back(x);
            p = end;
        }
    }
    if (v.size() != want) {
        std::fprintf(stderr, "refcuda_bench: %s needs %zu numbers\n", name, want);
        std::exit(2);
    }
    return v;
}

int fail(const char* what, cudaError_t e) {
    std::fprintf(stderr, "refcuda_bench: %s: %s\n", what, cudaGetErrorString(e));
    return 3;
}

}  // namespace

int main(int argc, char** argv) {
    const char* sL = opt(argc, argv, "--layers");
    const char* sN = opt(argc, argv, "--packets");
    const char* sK = opt(argc, argv, "--calls");
    if (!sL || !sN || !sK) {
        std::fprintf(stderr, "refcuda_bench: --layers, --packets and --calls are required\n");
        return 2;
    }
    const int L = std::atoi(sL);
    const long long N64 = std::atoll(sN);
    const int K = std::atoi(sK);
    // the reference's per-thread curand states: N/256 + 1 blocks of 256 threads
    // must fit in the RNGS-state array its first call allocates
    if (L < 1 || L > 64 || N64 < 1 || (N64 / 256 + 1) * 256 > (long long)RNGS || K < 1) {
        std::fprintf(stderr, "refcuda_bench: need 1 <= layers <= 64, 1 <= packets with "
                             "(packets/256 + 1) * 256 <= %d, calls >= 1\n", (int)RNGS);
        return 2;
    }
    const int N = (int)N64;
    std::vector<float> n = floats(opt(argc, argv, "-n"), L, "-n");
    std::vector<float> g = floats(opt(argc, argv, "-g"), L, "-g");
    std::vector<float> t = floats(opt(argc, argv, "-t"), L, "-t");
    std::vector<float> mua = floats(opt(argc, argv, "--mua"), L, "--mua");
    std::vector<float> mus = floats(opt(argc, argv, "--mus"), L, "--mus");
    std::vector<float> mut(L), bounds(L + 1, 0.0f);
    for (int i = 0; i < L; ++i) {
        mut[i] = mua[i] + mus[i];
        bounds[i + 1] = bounds[i] + t[i];
    }
    const bool R = opt(argc, argv, "--Rsphere") != nullptr;
    const bool T = opt(argc, argv, "--Tsphere") != nullptr;
    const float nanv = std::nanf("");
    std::vector<float> rs = R ? floats(opt(argc, argv, "--Rsphere"), 4, "--Rsphere")
                              : std::vector<float>(4, nanv);
    std::vector<float> ts = T ? floats(opt(argc, argv, "--Tsphere"), 4, "--Tsphere")
                              : std::vector<float>(4, nanv);
    const char* sRa = opt(argc, argv, "--Rangle");
    const char* sTa = opt(argc, argv, "--Tangle");
    const float R_angle = sRa ? (float)(std::atof(sRa) * M_PI / 180.0) : 0.0f;
    const float T_angle = sTa ? (float)(std::atof(sTa) * M_PI / 180.0) : 0.0f;
    const float R_f = rs[1] + rs[2] + rs[3], T_f = ts[1] + ts[2] + ts[3];
    const bool spec = false;

    // globals the reference's host code expects its program to create
    // (CUDA/ISMLMC.cu:82-85)
    rand_set = new bool[1]();
    globalDeviceStates = new curandState*[1];

    // ---- untimed warm-up through ISMLMC(): initialises the curand states for N
    float a0, a1, a2, a3, a4;
    thrust::tie(a0, a1, a2, a3, a4) =
        ISMLMC(0, N, L, n.data(), g.data(), t.data(), bounds.data(), mua.data(), mus.data(),
               mut.data(), R, rs[0], rs[1], rs[2], rs[3], R_f, R_angle, spec, T, ts[0], ts[1],
               ts[2], ts[3], T_f, T_angle);

    // ---- e2e: K calls of the reference's host entry point
    std::vector<double> e2e_s;
    double e2e_mean[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k < K; ++k) {
        const auto t0 = std::chrono::steady_clock::now();
        thrust::tie(a0, a1, a2, a3, a4) =
            ISMLMC(0, N, L, n.data(), g.data(), t.data(), bounds.data(), mua.data(), mus.data(),
                   mut.data(), R, rs[0], rs[1], rs[2], rs[3], R_f, R_angle, spec, T, ts[0], ts[1],
                   ts[2], ts[3], T_f, T_angle);
        const auto t1 = std::chrono::steady_clock::now();
        e2e_s.push_back(std::chrono::duration<double>(t1 - t0).count());
        const float m[5] = {a0, a1, a2, a3, a4};
        for (int j = 0; j < 5; ++j) e2e_mean[j] += m[j] / K;
    }

    // ---- kernel alone, on device-resident arrays, the launch shape of ISMLMC()
    cudaError_t e;
    float* d_arr[7] = {nullptr};
    const std::vector<float>* h_arr[7] = {&n, &g, &t, &bounds, &mua, &mus, &mut};
    for (int i = 0; i < 7; ++i) {
        const size_t bytes = h_arr[i]->size() * sizeof(float);
        if ((e = cudaMalloc(&d_arr[i], bytes)) != cudaSuccess) return fail("cudaMalloc", e);
        if ((e = cudaMemcpy(d_arr[i], h_arr[i]->data(), bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail("cudaMemcpy", e);
    }
    float* d_tally = nullptr;   // A, R_diffuse, R_specular, T_diffuse, T_direct
    if ((e = cudaMalloc(&d_tally, 5 * sizeof(float))) != cudaSuccess) return fail("cudaMalloc", e);
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    const int threads = 256, blocks = N / threads + 1;   // CUDAISMLMC.h:660-661
    std::vector<double> kern_s;
    double kern_mean[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k < K; ++k) {
        cudaMemsetAsync(d_tally, 0, 5 * sizeof(float), 0);
        cudaEventRecord(ev0, 0);
        CUDAISMLMC<<<blocks, threads>>>(globalDeviceStates[0], d_tally, d_tally + 1, d_tally + 2,
                                        d_tally + 3, d_tally + 4, N, L, d_arr[0], d_arr[1],
                                        d_arr[2], d_arr[3], d_arr[4], d_arr[5], d_arr[6], R, rs[0],
                                        rs[1], rs[2], rs[3], R_f, R_angle, spec, T, ts[0], ts[1],
                                        ts[2], ts[3], T_f, T_angle);
        cudaEventRecord(ev1, 0);
        if ((e = cudaEventSynchronize(ev1)) != cudaSuccess) return fail("kernel", e);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail("kernel launch", e);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        kern_s.push_back(ms / 1000.0);
        float h[5];
        if ((e = cudaMemcpy(h, d_tally, sizeof(h), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return fail("cudaMemcpy", e);
        for (int j = 0; j < 5; ++j) kern_mean[j] += h[j] / N / K;
    }
    int regs = -1;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, CUDAISMLMC) == cudaSuccess) regs = fa.numRegs;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, 0);

    auto list = [](const std::vector<double>& v) {
        std::string s = "[";
        char b[64];
        for (size_t i = 0; i < v.size(); ++i) {
            std::snprintf(b, sizeof b, "%s%.6f", i ? ", " : "", v[i]);
            s += b;
        }
        return s + "]";
    };
    std::printf("{\"packets_per_call\": %d, \"calls\": %d, \"threads\": %d, \"blocks\": %d, "
                "\"registers\": %d, \"gpu\": \"%s\", \"kernel_s\": %s, \"e2e_s\": %s, "
                "\"kernel_mean\": [%.7g, %.7g, %.7g, %.7g, %.7g], "
                "\"e2e_mean\": [%.7g, %.7g, %.7g, %.7g, %.7g]}\n",
                N, K, threads, blocks, regs, prop.name, list(kern_s).c_str(), list(e2e_s).c_str(),
                kern_mean[0], kern_mean[1], kern_mean[2], kern_mean[3], kern_mean[4], e2e_mean[0],
                e2e_mean[1], e2e_mean[2], e2e_mean[3], e2e_mean[4]);
    for (int i = 0; i < 7; ++i) cudaFree(d_arr[i]);
    cudaFree(d_tally);
    return 0;
}
