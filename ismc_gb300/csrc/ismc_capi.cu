// ismc_capi.cu -- host side of the C ABI declared in include/ismc.h.
//
// A context owns, on one device: a stream, capacity-grown device buffers
// (instances, prepared tables, packet ranges, queue prefix, tallies, queue
// head), pinned host staging for the host-pointer entry points, the tuned
// launch shape, and a CUDA graph of the whole host-pointer batch pipeline
// (H2D instances -> prepare -> prefix scan -> persistent propagate -> D2H
// tallies) that is replayed while the batch size and launch shape repeat.
// Compare CUDA/CUDAISMLMC.h:656-755, which allocates, copies, launches,
// synchronises and frees twelve buffers on every call.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include "ismc_dev.h"

struct ismc_ctx {
    int device = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    // device buffers (capacity in instances)
    uint32_t cap = 0;
    ismc_instance* d_in = nullptr;
    DevInst* d_inst = nullptr;
    DevRange* d_range = nullptr;
    unsigned long long* d_prefix = nullptr;
    ismc_tally* d_out = nullptr;
    unsigned long long* d_ctrl = nullptr;     // [0] queue head, [1] packets per chunk
    // pinned staging
    ismc_instance* h_in = nullptr;
    ismc_tally* h_out = nullptr;
    // launch shape
    ismc_tune tune{256, 0, 0, 0};
    uint32_t chunks_per_warp = 32;  // queue chunks per warp when sized on the device
    bool tuned = false;
    // graph of the host-pointer pipeline
    cudaGraphExec_t gexec = nullptr;
    uint32_t g_n = 0;
    ismc_tune g_tune{0, 0, 0, 0};
    uint32_t g_cpw = 0;
    uint32_t g_blocks = 0;
    char err[512] = {0};
};

static thread_local char g_lib_err[512];

static int set_err(ismc_ctx* c, int code, const char* fmt, ...) {
    char* buf = c ? c->err : g_lib_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, 512, fmt, ap);
    va_end(ap);
    return code;
}

int ismc_lib_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_lib_err, sizeof(g_lib_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return set_err(ctx, ISMC_ERR_CUDA, "%s failed: %s (%s:%d)", #call,           \
                           cudaGetErrorString(e_), __FILE__, __LINE__);                  \
    } while (0)

static const uint32_t kDefaultMaxEvents = 10000000u;

extern "C" int ismc_version(void) { return ISMC_ABI_VERSION; }

extern "C" size_t ismc_sizeof(int which) {
    switch (which) {
        case 0: return sizeof(ismc_stack);
        case 1: return sizeof(ismc_spheres);
        case 2: return sizeof(ismc_instance);
        case 3: return sizeof(ismc_tally);
        case 4: return sizeof(ismc_tune);
        case 5: return sizeof(ismc_solve_req);
        case 6: return sizeof(ismc_solve_out);
        default: return 0;
    }
}

static void release_buffers(ismc_ctx* c) {
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    cudaFree(c->d_in); cudaFree(c->d_inst); cudaFree(c->d_range); cudaFree(c->d_prefix);
    cudaFree(c->d_out);
    cudaFreeHost(c->h_in); cudaFreeHost(c->h_out);
    c->d_in = nullptr; c->d_inst = nullptr; c->d_range = nullptr; c->d_prefix = nullptr;
    c->d_out = nullptr; c->h_in = nullptr; c->h_out = nullptr;
    c->cap = 0;
}

static int ensure_capacity(ismc_ctx* ctx, uint32_t n) {
    if (n <= ctx->cap) return 0;
    uint32_t cap = std::max<uint32_t>(n, std::max<uint32_t>(64u, ctx->cap * 2u));
    release_buffers(ctx);
    CK(cudaMalloc(&ctx->d_in, sizeof(ismc_instance) * cap));
    CK(cudaMalloc(&ctx->d_inst, sizeof(DevInst) * cap));
    CK(cudaMalloc(&ctx->d_range, sizeof(DevRange) * cap));
    CK(cudaMalloc(&ctx->d_prefix, sizeof(unsigned long long) * (cap + 1)));
    CK(cudaMalloc(&ctx->d_out, sizeof(ismc_tally) * cap));
    CK(cudaMallocHost(&ctx->h_in, sizeof(ismc_instance) * cap));
    CK(cudaMallocHost(&ctx->h_out, sizeof(ismc_tally) * cap));
    ctx->cap = cap;
    return 0;
}

extern "C" int ismc_init(int device, ismc_ctx** out) {
    ismc_ctx* ctx = nullptr;
    if (!out) return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ismc_init: out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return set_err(nullptr, ISMC_ERR_NO_DEVICE, "ismc_init: no CUDA device (%s)",
                       cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ismc_init: device %d out of range [0,%d)",
                       device, ndev);
    ctx = new ismc_ctx();
    ctx->device = device;
    int rc = 0;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { rc = ISMC_ERR_CUDA; break; }
        if (cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
            rc = ISMC_ERR_CUDA; break;
        }
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            rc = ISMC_ERR_CUDA; break;
        }
        if (cudaMalloc(&ctx->d_ctrl, 2 * sizeof(unsigned long long)) != cudaSuccess) {
            rc = ISMC_ERR_CUDA; break;
        }
        int bps = 0;
        if (ismc_propagate_occupancy(256, &bps) != 0 || bps <= 0) { rc = ISMC_ERR_CUDA; break; }
    } while (0);
    if (rc) {
        set_err(nullptr, rc, "ismc_init: CUDA set-up failed on device %d: %s", device,
                cudaGetErrorString(cudaGetLastError()));
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        cudaFree(ctx->d_ctrl);
        delete ctx;
        return rc;
    }
    *out = ctx;
    return 0;
}

extern "C" int ismc_destroy(ismc_ctx* ctx) {
    if (!ctx) return ISMC_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    release_buffers(ctx);
    cudaFree(ctx->d_ctrl);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return 0;
}

extern "C" int ismc_last_error(const ismc_ctx* ctx, char* buf, size_t n) {
    if (!buf || n == 0) return ISMC_ERR_INVALID_ARG;
    const char* src = ctx ? ctx->err : g_lib_err;
    snprintf(buf, n, "%s", src);
    return 0;
}

// ---------------------------------------------------------------------------
// launch shape
// ---------------------------------------------------------------------------
static uint64_t total_packets(const ismc_instance* in, uint32_t n) {
    uint64_t t = 0;
    for (uint32_t i = 0; i < n; ++i) t += in[i].n_packets;
    return t;
}

// Resolve a (possibly partial) tune request into a concrete launch.  A zero
// chunk_packets is left zero: the scan kernel then sizes chunks on the device
// from the batch's total packet count (ctx->chunks_per_warp chunks per warp).
static int resolve_tune(ismc_ctx* ctx, const ismc_tune* req, ismc_tune* t, uint32_t* blocks) {
    ismc_tune x = req ? *req : ctx->tune;
    if (x.block_threads == 0) x.block_threads = ctx->tune.block_threads ? ctx->tune.block_threads : 256;
    if (x.block_threads % 32 || x.block_threads > 512)
        return set_err(ctx, ISMC_ERR_INVALID_ARG, "block_threads %u must be a multiple of 32 <= 512",
                       x.block_threads);
    int bps = 0;
    if (ismc_propagate_occupancy(x.block_threads, &bps) != 0 || bps <= 0)
        return set_err(ctx, ISMC_ERR_CUDA, "occupancy query failed for %u threads", x.block_threads);
    uint32_t want = x.blocks_per_sm ? std::min<uint32_t>(x.blocks_per_sm, (uint32_t)bps) : (uint32_t)bps;
    x.blocks_per_sm = want;
    if (x.max_events == 0) x.max_events = kDefaultMaxEvents;
    *t = x;
    *blocks = (uint32_t)ctx->sms * want;
    return 0;
}

// Launch shape of a batch with fewer packets than half the tuned launch's
// lanes: every packet its own lane, in full warps of 64-thread blocks spread
// over the SMs, one queue chunk (32 packets) per warp.  Under the tuned shape
// most warps would carry one or two live lanes yet issue every instruction,
// and the schedulers' issue slots would be shared by all of them; a small
// launch lasts as long as its longest packet, so its time per event is what
// counts.  Results do not depend on the launch shape.
static int small_batch_shape(ismc_ctx* ctx, uint64_t total, ismc_tune* t, uint32_t* blocks,
                             uint32_t* cpw) {
    const uint64_t lanes = (uint64_t)(*blocks) * t->block_threads;
    if (total == 0 || total * 2 > lanes) return 0;
    const uint32_t th = 64;
    int bps = 0;
    if (ismc_propagate_occupancy(th, &bps) != 0 || bps <= 0)
        return set_err(ctx, ISMC_ERR_CUDA, "occupancy query failed for %u threads", th);
    const uint64_t want = (total + th - 1) / th;
    *blocks = (uint32_t)std::min<uint64_t>(want, (uint64_t)ctx->sms * (uint32_t)bps);
    t->block_threads = th;
    t->blocks_per_sm = 0;
    *cpw = 1;
    return 0;
}

static int enqueue_pipeline(ismc_ctx* ctx, const ismc_instance* d_in, uint32_t n,
                            const ismc_tune& t, uint32_t blocks, uint32_t cpw, ismc_tally* d_out,
                            cudaStream_t s) {
    const uint32_t warps = blocks * (t.block_threads / 32);
    int rc = ismc_launch_prepare(d_in, n, ctx->d_inst, ctx->d_range, ctx->d_prefix, d_out,
                                 ctx->d_ctrl, t.chunk_packets, warps, cpw, (void*)s);
    if (rc) return set_err(ctx, rc, "prepare launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    PropParams p;
    p.inst = ctx->d_inst;
    p.range = ctx->d_range;
    p.chunk_prefix = ctx->d_prefix;
    p.tally = d_out;
    p.ctrl = ctx->d_ctrl;
    p.n_inst = n;
    p.max_events = t.max_events;
    rc = ismc_launch_propagate(p, blocks, t.block_threads, (void*)s);
    if (rc) return set_err(ctx, rc, "propagate launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}

// One instance's host-side check; the message goes to buf.  The prepare kernel
// (ismc_kernels.cu) makes the same checks on the device.
static int check_one(const ismc_instance& I, uint32_t i, char* buf, size_t nbuf) {
    const ismc_stack& S = I.stack;
    if (S.L < 1 || S.L > ISMC_MAXL) {
        snprintf(buf, nbuf, "instance %u: L=%u outside [1,%d]", i, S.L, ISMC_MAXL);
        return ISMC_ERR_INVALID_ARG;
    }
    if (I.mode > ISMC_MODE_PHYSICAL) {
        snprintf(buf, nbuf, "instance %u: unknown mode %u", i, I.mode);
        return ISMC_ERR_INVALID_ARG;
    }
    for (uint32_t l = 0; l < S.L; ++l) {
        if (!(S.n[l] > 0.0f) || !(S.d[l] > 0.0f) || !(S.mua[l] >= 0.0f) || !(S.mus[l] >= 0.0f) ||
            !(S.mut[l] >= 0.0f) || !(S.g[l] >= -1.0f && S.g[l] <= 1.0f) ||
            (S.mus[l] != 0.0f && !(S.mut[l] > 0.0f))) {
            snprintf(buf, nbuf,
                     "instance %u layer %u: need n>0, d>0, mua,mus,mut>=0, |g|<=1, mut>0 "
                     "when mus>0 (got n=%g d=%g mua=%g mus=%g mut=%g g=%g)",
                     i, l, S.n[l], S.d[l], S.mua[l], S.mus[l], S.mut[l], S.g[l]);
            return ISMC_ERR_INVALID_ARG;
        }
    }
    if (!(I.roulette_m >= 1.0f) || !(I.roulette_threshold >= 0.0f) ||
        !(I.roulette_threshold * I.roulette_m <= 1.0f)) {
        snprintf(buf, nbuf, "instance %u: roulette needs m >= 1 and 0 <= threshold * m <= 1 "
                            "(got threshold %g, m %g)", i, I.roulette_threshold, I.roulette_m);
        return ISMC_ERR_INVALID_ARG;
    }
    if (I.n_packets > ISMC_MAX_PACKETS) {
        snprintf(buf, nbuf, "instance %u: %llu packets exceed ISMC_MAX_PACKETS (2^31) of one "
                            "instance, beyond which 64-bit tallies could wrap; split it into "
                            "instances with consecutive packet_offset ranges",
                 i, (unsigned long long)I.n_packets);
        return ISMC_ERR_CAPACITY;
    }
    return 0;
}

static int check_instances(ismc_ctx* ctx, const ismc_instance* in, uint32_t n) {
    char msg[400];
    for (uint32_t i = 0; i < n; ++i) {
        const int rc = check_one(in[i], i, msg, sizeof msg);
        if (rc) return set_err(ctx, rc, "%s", msg);
    }
    return 0;
}

extern "C" int ismc_validate(const ismc_instance* inst, uint32_t n_inst, int32_t* status) {
    if (!inst && n_inst)
        return set_err(nullptr, ISMC_ERR_INVALID_ARG, "validate: inst is NULL");
    char msg[400];
    int first = 0;
    for (uint32_t i = 0; i < n_inst; ++i) {
        const int rc = check_one(inst[i], i, msg, sizeof msg);
        if (status) status[i] = rc;
        if (rc && !first) first = set_err(nullptr, rc, "%s", msg);
    }
    return first;
}

extern "C" int ismc_run_batch_device(ismc_ctx* ctx, const ismc_instance* d_inst, uint32_t n_inst,
                                     const ismc_tune* tune, ismc_tally* d_out, void* stream) {
    if (!ctx) return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ctx is NULL");
    if (!d_inst || !d_out || n_inst == 0)
        return set_err(ctx, ISMC_ERR_INVALID_ARG, "run_batch_device: null pointer or empty batch");
    CK(cudaSetDevice(ctx->device));
    int rc = ensure_capacity(ctx, n_inst);
    if (rc) return rc;
    ismc_tune t;
    uint32_t blocks;
    rc = resolve_tune(ctx, tune, &t, &blocks);
    if (rc) return rc;
    // the caller's stream exactly as given (NULL = the legacy default stream),
    // so the launch is ordered with the caller's own copies and events
    return enqueue_pipeline(ctx, d_inst, n_inst, t, blocks, ctx->chunks_per_warp, d_out,
                            (cudaStream_t)stream);
}

static bool same_tune(const ismc_tune& a, const ismc_tune& b) {
    return a.block_threads == b.block_threads && a.blocks_per_sm == b.blocks_per_sm &&
           a.chunk_packets == b.chunk_packets && a.max_events == b.max_events;
}

extern "C" int ismc_run_batch(ismc_ctx* ctx, const ismc_instance* inst, uint32_t n_inst,
                              const ismc_tune* tune, ismc_tally* out) {
    if (!ctx) return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ctx is NULL");
    if (!inst || !out || n_inst == 0)
        return set_err(ctx, ISMC_ERR_INVALID_ARG, "run_batch: null pointer or empty batch");
    int rc = check_instances(ctx, inst, n_inst);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    rc = ensure_capacity(ctx, n_inst);
    if (rc) return rc;
    ismc_tune t;
    uint32_t blocks;
    rc = resolve_tune(ctx, tune, &t, &blocks);
    if (rc) return rc;
    uint32_t cpw = ctx->chunks_per_warp;
    if (!tune || tune->block_threads == 0) {
        rc = small_batch_shape(ctx, total_packets(inst, n_inst), &t, &blocks, &cpw);
        if (rc) return rc;
    }
    memcpy(ctx->h_in, inst, sizeof(ismc_instance) * n_inst);
    // replay the captured pipeline when batch size and launch shape repeat
    if (!(ctx->gexec && ctx->g_n == n_inst && same_tune(ctx->g_tune, t) && ctx->g_cpw == cpw &&
          ctx->g_blocks == blocks)) {
        if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemcpyAsync(ctx->d_in, ctx->h_in, sizeof(ismc_instance) * n_inst,
                        cudaMemcpyHostToDevice, ctx->stream);
        int rc2 = enqueue_pipeline(ctx, ctx->d_in, n_inst, t, blocks, cpw, ctx->d_out, ctx->stream);
        cudaMemcpyAsync(ctx->h_out, ctx->d_out, sizeof(ismc_tally) * n_inst,
                        cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (rc2) { if (g) cudaGraphDestroy(g); return rc2; }
        if (e != cudaSuccess)
            return set_err(ctx, ISMC_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&ctx->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess)
            return set_err(ctx, ISMC_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
        ctx->g_n = n_inst;
        ctx->g_tune = t;
        ctx->g_cpw = cpw;
        ctx->g_blocks = blocks;
    }
    CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    memcpy(out, ctx->h_out, sizeof(ismc_tally) * n_inst);
    return 0;
}

extern "C" int ismc_run(ismc_ctx* ctx, const ismc_stack* stack, const ismc_spheres* sph,
                        uint64_t n_packets, uint64_t seed, uint32_t mode, ismc_tally* out) {
    if (!ctx) return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ctx is NULL");
    if (!stack || !sph || !out) return set_err(ctx, ISMC_ERR_INVALID_ARG, "run: null pointer");
    ismc_instance in;
    memset(&in, 0, sizeof(in));
    in.stack = *stack;
    in.spheres = *sph;
    in.n_packets = n_packets;
    in.packet_offset = 0;
    in.seed = seed;
    in.stream = 0;
    in.mode = mode;
    in.roulette_threshold = 1e-4f;   // MLMC.py:86
    in.roulette_m = 10.0f;           // MLMC.py:87
    int rc = ismc_run_batch(ctx, &in, 1, nullptr, out);
    if (rc) return rc;
    if (out->status) return set_err(ctx, out->status, "run: instance status %d", out->status);
    return 0;
}

// ---------------------------------------------------------------------------
// autotuner: time short trial launches of a scaled-down copy of the batch
// ---------------------------------------------------------------------------
extern "C" int ismc_autotune(ismc_ctx* ctx, const ismc_instance* inst, uint32_t n_inst,
                             ismc_tune* out) {
    if (!ctx) return set_err(nullptr, ISMC_ERR_INVALID_ARG, "ctx is NULL");
    if (!inst || n_inst == 0) return set_err(ctx, ISMC_ERR_INVALID_ARG, "autotune: empty batch");
    int rc = check_instances(ctx, inst, n_inst);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    // trial batch: the same instances with budgets scaled to ~4e6 packets total
    const uint64_t total = std::max<uint64_t>(1, total_packets(inst, n_inst));
    const double scale = std::min(1.0, 4.0e6 / (double)total);
    std::vector<ismc_instance> trial(inst, inst + n_inst);
    for (auto& x : trial) x.n_packets = (uint64_t)((double)x.n_packets * scale + 0.5);
    rc = ensure_capacity(ctx, n_inst);
    if (rc) return rc;
    CK(cudaMemcpy(ctx->d_in, trial.data(), sizeof(ismc_instance) * n_inst, cudaMemcpyHostToDevice));
    // events are destroyed and the context's chunking restored on every exit path
    struct Trial {
        ismc_ctx* c;
        uint32_t saved_cpw;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Trial() {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            c->chunks_per_warp = saved_cpw;
        }
    } tr{ctx, ctx->chunks_per_warp};
    CK(cudaEventCreate(&tr.e0));
    CK(cudaEventCreate(&tr.e1));
    const uint32_t threads_c[] = {128, 256, 512};
    const uint32_t cpw_c[] = {8, 32, 128};
    float best = 1e30f;
    ismc_tune best_t = ctx->tune;
    uint32_t best_cpw = ctx->chunks_per_warp;
    for (uint32_t th : threads_c) {
        for (uint32_t cpw : cpw_c) {
            ismc_tune t{th, 0, 0, 0};
            ismc_tune r;
            uint32_t blocks;
            if (resolve_tune(ctx, &t, &r, &blocks)) continue;
            ctx->chunks_per_warp = cpw;
            float best_ms = 1e30f;
            for (int rep = 0; rep < 2; ++rep) {
                CK(cudaEventRecord(tr.e0, ctx->stream));
                rc = enqueue_pipeline(ctx, ctx->d_in, n_inst, r, blocks, cpw, ctx->d_out, ctx->stream);
                if (rc) return rc;
                CK(cudaEventRecord(tr.e1, ctx->stream));
                CK(cudaEventSynchronize(tr.e1));
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, tr.e0, tr.e1));
                best_ms = std::min(best_ms, ms);
            }
            if (best_ms < best) { best = best_ms; best_t = t; best_cpw = cpw; }
        }
    }
    tr.saved_cpw = best_cpw;
    // keep the winning block size and chunks-per-warp; the chunk size itself is
    // re-derived on the device from each batch's total packet count
    ctx->tune.block_threads = best_t.block_threads;
    ctx->tune.blocks_per_sm = 0;
    ctx->chunks_per_warp = best_cpw;
    ctx->tuned = true;
    if (out) *out = ctx->tune;
    return 0;
}
