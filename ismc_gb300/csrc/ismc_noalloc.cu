// ismc_noalloc.cu -- batch entry point that allocates no GPU memory.
//
// Who needs it: code that is not allowed to call cudaMalloc -- for example a
// plugin running inside a host application that owns every byte of device
// memory through its own pool, a caller with a hard memory budget that must
// not grow, or a latency-critical loop that cannot afford the implicit
// synchronisation an allocation can cause.  Such a caller already holds its
// input instances and output tallies in device memory it manages; this entry
// point needs nothing else.
//
// The working memory that ismc_run_batch_device takes from a context (prepared
// tables, packet ranges, work-queue prefix, queue head and chunk size) lives
// here in one file-scope __device__ array of fixed size, sized for at most
// ISMC_NOALLOC_MAX_INST instances (about 1.2 MB).  Every GPU that loads the
// library keeps that array until the process exits.
#include <cuda.h>          // CUcontext / CUresult types only; the driver calls go
                           // through cudaGetDriverEntryPointByVersion, no -lcuda
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include "ismc_dev.h"

namespace {

struct NoallocScratch {
    DevInst inst[ISMC_NOALLOC_MAX_INST];
    DevRange range[ISMC_NOALLOC_MAX_INST];
    unsigned long long prefix[ISMC_NOALLOC_MAX_INST + 1];
    unsigned long long ctrl[2];
};

}  // namespace

// The array itself.  Host code must not pass this name to a kernel: on the
// host it is only a stand-in, and its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char ismc_noalloc_scratch[sizeof(NoallocScratch)];

namespace {

// A __device__ array has one address per CUDA context that loaded the
// library's module, not per device: a host application may make its own
// driver-API context current, and cudaDeviceReset replaces the primary
// context (and the array's address) with a new one.  The looked-up address is
// therefore cached per context, keyed by the context's process-unique ID.
constexpr int kMaxContexts = 64;

struct ContextSetup {
    unsigned long long ctx_id = 0;
    int sms = 0;
    NoallocScratch* scratch = nullptr;   // device address of ismc_noalloc_scratch
};

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

std::mutex g_setup_mu;
ContextSetup g_setup[kMaxContexts];
int g_n_setup = 0, g_next_slot = 0;
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

int resolve_driver_calls() {
    if (g_ctx_get_current && g_ctx_get_id) return 0;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                      cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                                      cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: cuCtxGetCurrent / cuCtxGetId "
                                             "unavailable from the driver");
    g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
    g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f2);
    return 0;
}

// Once per CUDA context, with that context current: look up the array's
// device address in it and the device's SM count.  A thread with no current
// context gets the device's primary context, which the runtime's first call
// (cudaGetSymbolAddress) creates and makes current.
int context_setup(int dev, ContextSetup* out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    int rc = resolve_driver_calls();
    if (rc) return rc;
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: cuCtxGetCurrent failed");
    void* p = nullptr;
    if (!c) {
        const cudaError_t e = cudaGetSymbolAddress(&p, ismc_noalloc_scratch);
        if (e != cudaSuccess)
            return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: cudaGetSymbolAddress failed: %s",
                                  cudaGetErrorString(e));
        if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c)
            return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: no current CUDA context");
    }
    unsigned long long id = 0;
    if (g_ctx_get_id(c, &id) != CUDA_SUCCESS)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: cuCtxGetId failed");
    for (int k = 0; k < g_n_setup; ++k) {
        if (g_setup[k].ctx_id == id) {
            *out = g_setup[k];   // a copy: the table entry may be reused later
            return 0;
        }
    }
    cudaError_t e = cudaGetSymbolAddress(&p, ismc_noalloc_scratch);
    if (e != cudaSuccess)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: cudaGetSymbolAddress failed: %s",
                              cudaGetErrorString(e));
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || sms <= 0)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: SM count query failed: %s",
                              cudaGetErrorString(e));
    // a bounded table: past kMaxContexts contexts (each cudaDeviceReset makes
    // a new one) the oldest entry is reused
    const int slot = g_n_setup < kMaxContexts ? g_n_setup++ : g_next_slot;
    if (g_n_setup == kMaxContexts) g_next_slot = (slot + 1) % kMaxContexts;
    g_setup[slot].ctx_id = id;
    g_setup[slot].scratch = static_cast<NoallocScratch*>(p);
    g_setup[slot].sms = sms;
    *out = g_setup[slot];
    return 0;
}

}  // namespace

extern "C" int ismc_run_batch_noalloc(const ismc_instance* d_inst, uint32_t n_inst,
                                      const ismc_tune* tune, ismc_tally* d_out, void* stream) {
    if (!d_inst || !d_out || n_inst == 0)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG, "run_batch_noalloc: null pointer or empty batch");
    if (n_inst > ISMC_NOALLOC_MAX_INST)
        return ismc_lib_error(ISMC_ERR_CAPACITY,
                              "run_batch_noalloc: %u instances exceed the fixed capacity of %d; "
                              "split the batch or use ismc_run_batch_device",
                              n_inst, ISMC_NOALLOC_MAX_INST);
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return ismc_lib_error(ISMC_ERR_NO_DEVICE, "run_batch_noalloc: no current CUDA device: %s",
                              cudaGetErrorString(e));
    ContextSetup setup;
    int rc = context_setup(dev, &setup);
    if (rc) return rc;
    const ContextSetup* d = &setup;

    const uint32_t threads = (tune && tune->block_threads) ? tune->block_threads : 256u;
    if (threads % 32 || threads > 512)
        return ismc_lib_error(ISMC_ERR_INVALID_ARG,
                              "run_batch_noalloc: block_threads %u must be a multiple of 32 <= 512",
                              threads);
    int bps = 0;
    if (ismc_propagate_occupancy(threads, &bps) != 0 || bps <= 0)
        return ismc_lib_error(ISMC_ERR_CUDA, "run_batch_noalloc: occupancy query failed");
    const uint32_t per_sm = (tune && tune->blocks_per_sm) ? std::min<uint32_t>(tune->blocks_per_sm, (uint32_t)bps)
                                                          : (uint32_t)bps;
    const uint32_t blocks = (uint32_t)d->sms * per_sm;
    const uint32_t warps = blocks * (threads / 32);
    NoallocScratch* S = d->scratch;
    // the prepare and scan kernels rewrite every scratch word the propagator
    // reads (tables, ranges, prefix, queue head, chunk size) and zero the
    // caller's tallies, so nothing left from an earlier call is used
    // 32 queue chunks per warp when the chunk size is left to the device: the
    // context entry points' default, which shortens the end-of-launch tail
    rc = ismc_launch_prepare(d_inst, n_inst, S->inst, S->range, S->prefix, d_out, S->ctrl,
                             tune ? tune->chunk_packets : 0u, warps, 32u, stream);
    if (rc)
        return ismc_lib_error(rc, "run_batch_noalloc: prepare launch failed: %s",
                              cudaGetErrorString(cudaGetLastError()));
    PropParams p;
    p.inst = S->inst;
    p.range = S->range;
    p.chunk_prefix = S->prefix;
    p.tally = d_out;
    p.ctrl = S->ctrl;
    p.n_inst = n_inst;
    p.max_events = (tune && tune->max_events) ? tune->max_events : 10000000u;
    rc = ismc_launch_propagate(p, blocks, threads, stream);
    if (rc)
        return ismc_lib_error(rc, "run_batch_noalloc: propagate launch failed: %s",
                              cudaGetErrorString(cudaGetLastError()));
    return 0;
}
