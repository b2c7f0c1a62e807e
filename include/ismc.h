/*
 * ismc.h -- C ABI of the GB300 integrating-sphere Monte Carlo propagator.
 *
 * This is the boundary the reference's forward model is replaced behind.  The
 * reference exposes its forward model three ways, all of which map onto the
 * entry points below:
 *
 *   ISMC.py:164-406      ISMC(N, n, g, t, mu_a, mu_s, mu_t, R, R_pw, ..., T_angle)
 *                        -> (A, R_d, R_s, T_d, T_u) as fractions of N  (one slab)
 *   ISMLMC.py:101-347    ISMLMC(...) with list-valued n/g/t/mu_a/mu_s/mu_t (stack)
 *   CUDA/CUDAISMLMC.h:656-755
 *                        thrust::tuple<float x5> ISMLMC(int dev, int N, int layers,
 *                        float* n, float* g, float* t, float* bounds, float* mu_a,
 *                        float* mu_s, float* mu_t, bool R, float R_pw, ...)
 *
 * Conventions
 *   - Plain C, fixed-width types, natural alignment, no packing pragmas: every
 *     struct below has explicit padding so its layout is the same for C, C++,
 *     ctypes and any other FFI.
 *   - Every entry point returns 0 on success or a negative ISMC_ERR_* code.
 *     Nothing calls exit() (contrast CUDA/CUDAISMLMC.h:41-48).  The text of the
 *     last error of a context is available from ismc_last_error().
 *   - Caller owns every host array it passes; nothing is retained after return.
 *   - A context owns its device buffers, stream and graphs.  One context must
 *     not be used from two threads at once without an external lock; separate
 *     contexts are independent (no global mutable state in the library).
 *   - Results are integer fixed-point sums (scale 2^-scale_log2 per unit of
 *     packet weight), so a given (seed, stream, packet range) is bit-identical
 *     for any launch shape, chunking or sharding.
 */
#ifndef ISMC_GB300_H
#define ISMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ISMC_ABI_VERSION 1
#define ISMC_MAXL 16            /* max layers in a stack (slides count as layers) */

/* error codes */
#define ISMC_OK 0
#define ISMC_ERR_INVALID_ARG   (-1)
#define ISMC_ERR_CUDA          (-2)
#define ISMC_ERR_STEP_LIMIT    (-3)   /* some packet exceeded the per-packet event cap */
#define ISMC_ERR_NO_DEVICE     (-4)
#define ISMC_ERR_ALLOC         (-5)
#define ISMC_ERR_CAPACITY      (-6)   /* request beyond a fixed capacity: a fixed-size
                                         buffer, or ISMC_MAX_PACKETS per instance */
#define ISMC_ERR_INTERNAL      (-7)

/* propagation modes */
#define ISMC_MODE_COMPAT   0u   /* reproduce ISMC.py / ISMLMC.py+MLMC.MC semantics */
#define ISMC_MODE_PHYSICAL 1u   /* physically consistent slides / re-incidence */

/* tally order (index into ismc_tally.sum / sumsq) -- the reference's return order */
#define ISMC_T_A   0
#define ISMC_T_RD  1
#define ISMC_T_RS  2
#define ISMC_T_TD  3
#define ISMC_T_TU  4

/*
 * A layer stack, top (index 0, facing the R sphere) to bottom.  A layer with
 * mus == 0 is a non-scattering slide ("glass"), as in ISMLMC.py:81 and
 * MLMC.py:97.  mut is the interaction coefficient the walk uses
 * (the reference's callers pass mu_a + mu_s: lookup.py:238, minimization.py:205).
 * Units: 1/cm and cm.  The ambient index is 1 on both sides.
 */
typedef struct ismc_stack {
    uint32_t L;
    uint32_t _pad0;
    float n[ISMC_MAXL];
    float mua[ISMC_MAXL];
    float mus[ISMC_MAXL];
    float mut[ISMC_MAXL];
    float g[ISMC_MAXL];
    float d[ISMC_MAXL];
} ismc_stack;

/*
 * Sphere geometry with the reference's argument meaning (ISMC.py:164-165):
 * R/T = sphere present; pw = wall reflectance; fs/fp/fd = sample, source
 * (R) or optional (T) port and detector AREA fractions; f = total port
 * fraction; *_angle = acceptance half-angle in RADIANS used when that sphere
 * is absent (ISMC.py:221-236); specular_included tilts the beam to mu_z=0.99
 * (ISMC.py:177-179).
 */
typedef struct ismc_spheres {
    uint8_t R, T, specular_included, _pad0[5];
    double R_pw, R_fs, R_fp, R_fd, R_f, R_angle;
    double T_pw, T_fs, T_fp, T_fd, T_f, T_angle;
} ismc_spheres;

/*
 * Largest packet count of one instance: 2^31.  Tallies are 64-bit sums of
 * per-packet scores quantised to 2^-32 (ismc_tally), and a packet's scored
 * weights add up to 1 on average (roulette_threshold * roulette_m <= 1 keeps
 * every single score near that), so 2^31 packets use at most about half of
 * the 2^64 range of any sum or sum of squares.  A larger simulation is split
 * into instances with consecutive packet_offset ranges; their tallies add
 * exactly, in wider than 64-bit arithmetic once the total passes 2^31
 * packets (the Python API's Engine.run_batch does this split and sum).
 * Instances beyond the limit are refused with ISMC_ERR_CAPACITY instead of
 * returning wrapped sums.
 */
#define ISMC_MAX_PACKETS 2147483648ull

/* One simulation instance of a batch. */
typedef struct ismc_instance {
    ismc_stack stack;
    ismc_spheres spheres;
    uint64_t n_packets;       /* packets to launch, at most ISMC_MAX_PACKETS */
    uint64_t packet_offset;   /* id of the first packet (sharding / resume) */
    uint64_t seed;            /* Philox key */
    uint32_t stream;          /* Philox stream id (independent streams per seed) */
    uint32_t mode;            /* ISMC_MODE_* */
    float roulette_threshold; /* 1e-4 as in MLMC.py:86, 1e-3 as in ISMC.py:136 */
    float roulette_m;         /* survival 1/m, weight *m (10 in the reference);
                                 m >= 1 and roulette_threshold * m <= 1 */
} ismc_instance;

/*
 * Result of one instance.  sum[k] = sum over packets of round(x_k * 2^scale_log2)
 * and sumsq[k] = sum of round(x_k^2 * 2^scale_log2), where x_k is the packet's
 * weight scored into tally k (ISMC_T_*).  Fractions of N as the reference
 * returns them (ISMC.py:406) are sum[k] / (n * 2^scale_log2).
 */
typedef struct ismc_tally {
    uint64_t n;               /* packets simulated */
    uint64_t sum[5];
    uint64_t sumsq[5];
    uint64_t steps;           /* free-path draws in scattering layers */
    uint64_t events;          /* propagation events (steps, boundary hits, incidences) */
    uint64_t reincidences;    /* sphere re-incidences */
    uint64_t capped;          /* packets stopped by the event cap */
    uint64_t trapped;         /* packets refracted into a slide at a direction that
                                 both faces totally reflect (a rounding artefact of
                                 near-grazing entry, ~1e-7 per entry): their weight
                                 is dropped instead of bouncing forever */
    uint32_t scale_log2;
    int32_t status;           /* ISMC_OK, ISMC_ERR_STEP_LIMIT, or (instance not run, n = 0)
                                 ISMC_ERR_INVALID_ARG / ISMC_ERR_CAPACITY */
    float analytic_specular;  /* deterministic specular reflectance of the stack (see ismc_run) */
    float analytic_ballistic; /* deterministic unscattered transmittance (normal incidence) */
} ismc_tally;

/* Launch tuning; pass NULL to use the context's autotuned choice. */
typedef struct ismc_tune {
    uint32_t block_threads;   /* threads per block (multiple of 32, <= 512) */
    uint32_t blocks_per_sm;   /* resident blocks per SM requested (0 = occupancy max) */
    uint32_t chunk_packets;   /* packets a warp claims from the work queue at once */
    uint32_t max_events;      /* per-packet event cap (0 = default 10,000,000) */
} ismc_tune;

typedef struct ismc_ctx ismc_ctx;

/* ABI version (ISMC_ABI_VERSION). */
int ismc_version(void);

/* Create a context on a CUDA device.  Replaces the per-call cudaSetDevice +
 * curand state set-up of CUDA/CUDAISMLMC.h:660-683. */
int ismc_init(int device, ismc_ctx** out);

/* Release a context and everything it owns. */
int ismc_destroy(ismc_ctx* ctx);

/*
 * One forward simulation: replaces ISMC.py:164 ISMC() / ISMLMC.py:101 ISMLMC()
 * and the CUDA host wrapper CUDA/CUDAISMLMC.h:656 ISMLMC().  The reference's
 * roulette threshold of MLMC.py:86 (1e-4) and m = 10 are used; for the single
 * slab driver's 1e-3 (ISMC.py:136) use ismc_run_batch with one instance.
 * Host pointers in, host tally out; blocks until the result is ready.
 */
int ismc_run(ismc_ctx* ctx, const ismc_stack* stack, const ismc_spheres* sph,
             uint64_t n_packets, uint64_t seed, uint32_t mode, ismc_tally* out);

/*
 * Many independent simulations of uneven size in one persistent launch,
 * drained from a device work queue.  Replaces the per-grid-point loop of
 * CUDA/ISMLMC-lookup.cu:153-421 (singleLayerSampleSpace), lookup.py:228-259
 * (sample_space) and the per-objective launches of
 * CUDA/ISMLMC-minimization.cu:89-131 (cost).  out has n_inst entries.
 * With tune NULL (or block_threads 0), a batch of fewer packets than half the
 * tuned launch's lanes runs one packet per lane in 64-thread blocks; the
 * tallies do not depend on the launch shape.
 */
int ismc_run_batch(ismc_ctx* ctx, const ismc_instance* inst, uint32_t n_inst,
                   const ismc_tune* tune, ismc_tally* out);

/*
 * Device-pointer variant for callers whose instances are already resident on
 * the GPU: d_inst and d_out are device pointers (n_inst entries), stream is the
 * cudaStream_t to launch on, used as given (NULL = the legacy default stream).
 * Asynchronous: returns after enqueueing.  The context's device buffers are
 * reused by the next call, so calls on one context must not overlap on the GPU
 * (enqueue them on one stream).  Used for graph capture and by callers that
 * keep data in HBM.
 */
int ismc_run_batch_device(ismc_ctx* ctx, const ismc_instance* d_inst, uint32_t n_inst,
                          const ismc_tune* tune, ismc_tally* d_out, void* stream);

/*
 * Batch entry point that allocates no GPU memory (no counterpart in the
 * reference, which allocates and frees on every call).  For callers that may
 * not call cudaMalloc: a plugin inside an application that owns all device
 * memory, a fixed memory budget, or a loop that cannot take an allocation's
 * implicit synchronisation.  Inputs and outputs are the caller's device
 * pointers, as for ismc_run_batch_device; the library's working memory is one
 * fixed __device__ array sized for ISMC_NOALLOC_MAX_INST instances (~1.2 MB,
 * kept by every GPU that loads the library until the process exits).
 *   - Needs no context; runs on the calling thread's current device and on
 *     `stream` as given (NULL = legacy default stream).
 *   - The array has one address per CUDA context.  The first call in each
 *     context (the device's primary context, a driver-API context the caller
 *     made current, or the new primary context after cudaDeviceReset) looks
 *     that address up; make that first call before any stream capture.
 *   - n_inst > ISMC_NOALLOC_MAX_INST returns ISMC_ERR_CAPACITY (message in
 *     ismc_last_error(NULL, ...)).
 *   - All calls share the one array: calls that overlap on the GPU (different
 *     streams, or different host threads) race and corrupt each other.
 *     Serialise them, e.g. on one stream.  Each call re-initialises everything
 *     it reads, so results never depend on an earlier call.
 */
#define ISMC_NOALLOC_MAX_INST 1024
int ismc_run_batch_noalloc(const ismc_instance* d_inst, uint32_t n_inst, const ismc_tune* tune,
                           ismc_tally* d_out, void* stream);

/*
 * Host-side check of a batch, no GPU needed: the checks ismc_run_batch makes
 * before it launches anything (layer parameters, mode, roulette, and
 * n_packets <= ISMC_MAX_PACKETS).  status (n_inst entries, may be NULL)
 * receives ISMC_OK, ISMC_ERR_INVALID_ARG or ISMC_ERR_CAPACITY per instance;
 * the return value is the first instance's error, its text in
 * ismc_last_error(NULL, ...).  The device-pointer entry points make the same
 * checks on the GPU and report them in each tally's status.
 */
int ismc_validate(const ismc_instance* inst, uint32_t n_inst, int32_t* status);

/* Choose block size / chunk size for a representative batch by timing short
 * trial launches; the choice is stored in the context and returned in *out. */
int ismc_autotune(ismc_ctx* ctx, const ismc_instance* inst, uint32_t n_inst,
                  ismc_tune* out);

/* Copy the last error message of ctx (or of the library when ctx is NULL). */
int ismc_last_error(const ismc_ctx* ctx, char* buf, size_t n);

/* ------------------------------------------------------------------------
 * Inverse solver (plain path): PRAXIS minimisation of the reference's cost
 *   sqrt( ((R_d-M_R)/M_R)^2 + (R_s-M_S)^2 + ((T_d-M_T)/M_T)^2 + (T_u-M_U)^2 )
 * over (mu_a, mu_s') of one layer, each objective a GPU Monte Carlo run
 * (minimization.py:201-238, CUDA/ISMLMC-minimization.cu:89-131 and :476).
 * Many solves advance in lockstep: every round of objective evaluations of all
 * active solves is ONE batched launch.
 * ------------------------------------------------------------------------ */
typedef struct ismc_solve_req {
    ismc_instance base;       /* stack, spheres, packets per objective, seed, mode, roulette */
    uint32_t layer;           /* layer whose (mu_a, mu_s') are unknown; its g is kept */
    uint32_t separate;        /* 1: R-only, T-only and sphere-less runs per objective
                                 (minimization.py:209-225); 0: one run with both spheres */
    uint32_t log_coords;      /* 1: minimise over (ln mu_a, ln mu_s'); 0: over (mu_a, mu_s') */
    uint32_t max_evals;       /* objective evaluations per minimisation (0 = 2000) */
    uint32_t max_restarts;    /* re-runs when the result leaves the box (minimization.py:260-271) */
    uint32_t fresh_streams;   /* 0: every evaluation of a solve reuses its Philox stream (common
                                 random numbers, a deterministic objective); 1: a new stream per
                                 evaluation, like the reference's global random state */
    uint32_t max_refits;      /* re-runs of a minimisation that stopped short (0: none).  PRAXIS
                                 stops after two iterations without progress, which a rough
                                 Monte Carlo objective can cause far from the minimum.  An end
                                 point inside the box whose cost exceeds 5x the objective's own
                                 Monte Carlo standard error is probed 3 % either side along each
                                 axis; a probe 10 % lower starts a re-run from it.  Not for
                                 minimisations stopped by max_evals. */
    uint32_t _pad0;
    double meas[4];           /* measured R_d, R_s, T_d, T_u; NaN = not measured */
    double x0[2];             /* initial (mu_a, mu_s') */
    double lo[2], hi[2];      /* accepted box for (mu_a, mu_s'): answers outside it are
                                 re-run (max_restarts); the objective is evaluated only
                                 inside it, widened to take in an x0 that lies outside */
    double h0, t0;            /* PRAXIS initial step and tolerance (in the chosen coordinates) */
} ismc_solve_req;

typedef struct ismc_solve_out {
    double x[2];              /* recovered (mu_a, mu_s') */
    double cost;              /* objective at x (last evaluation there) */
    uint32_t evals;           /* objective evaluations, all restarts included */
    uint32_t restarts;
    int32_t status;           /* ISMC_OK, or ISMC_ERR_CAPACITY when every restart left the box */
    uint32_t rounds;          /* batched launches this solve took part in */
    uint32_t refits;          /* re-runs after a minimisation stopped short (max_refits) */
    uint32_t _pad0;
} ismc_solve_out;

/* Solve n independent inverse problems; out has n entries. */
int ismc_solve_batch(ismc_ctx* ctx, const ismc_solve_req* req, uint32_t n,
                     ismc_solve_out* out);

/* PRAXIS on a host callback, no GPU involved (n <= 8 variables).  Returns the
 * minimum in *fmin and the number of evaluations in *nevals. */
typedef double (*ismc_objective)(const double* x, int n, void* user);
int ismc_praxis(ismc_objective f, void* user, int n, double* x, double t0, double h0,
                int maxfun, double* fmin, int* nevals);

/* ------------------------------------------------------------------------
 * Surrogate network (no counterpart in the reference): MLP
 * 5 -> 256 -> 256 -> 256 -> 6, SiLU, BF16 weights/activations, FP32
 * accumulation on the tcgen05 tensor cores, Adam, Gaussian negative
 * log-likelihood.  Inputs per row: (ln mu_a, ln mu_s', g, d, n), mapped
 * internally from [ln .01, ln 10] x [ln 1, ln 100] x [.6, .95] x [.02, .5] x
 * [1.33, 1.5] to [-1, 1]; outputs per row: means of (R_d, T_d, T_u) and their
 * log-variances.  All array arguments are DEVICE pointers, row-major fp32;
 * batch sizes are multiples of 128.  Parameters are flattened as
 * W1[256x5], b1, W2[256x256], b2, W3[256x256], b3, W4[6x256], b4.
 * ------------------------------------------------------------------------ */
typedef struct ismc_mlp ismc_mlp;
int ismc_mlp_create(int device, uint32_t max_batch, uint64_t seed, ismc_mlp** out);
int ismc_mlp_destroy(ismc_mlp* m);
size_t ismc_mlp_nparam(void);
int ismc_mlp_get_params(ismc_mlp* m, float* host, size_t n);        /* host array */
int ismc_mlp_set_params(ismc_mlp* m, const float* host, size_t n);  /* resets Adam */
int ismc_mlp_forward(ismc_mlp* m, const float* d_x, uint32_t batch, float* d_out);
int ismc_mlp_grad(ismc_mlp* m, const float* d_x, const float* d_y, uint32_t batch,
                  float* d_grad, float* loss /* host, may be NULL */);
int ismc_mlp_train_step(ismc_mlp* m, const float* d_x, const float* d_y, uint32_t batch,
                        float lr, float* loss /* host; NULL = do not wait */);
int ismc_mlp_train_epoch(ismc_mlp* m, const float* d_x, const float* d_y, uint32_t n_rows,
                         uint32_t batch, const float* lrs /* host, n_rows/batch */,
                         float* loss /* host, last batch, may be NULL */);
int ismc_mlp_sync(ismc_mlp* m);
int ismc_mlp_gemm_test(ismc_mlp* m, const void* d_a, const void* d_b, float* d_d, int M, int N,
                       int K, int splits);   /* D = A B^T, bf16 K-major operands, for tests */
int ismc_mlp_last_error(const ismc_mlp* m, char* buf, size_t n);
/* Polls each tensor-core pipeline wait makes before it gives up (default
 * 4194304, seconds at most).  A wait that runs out records an error that the
 * next synchronising call returns as ISMC_ERR_INTERNAL; the block first lets
 * its own tile copies and MMAs finish and frees its TMEM, so the context stays
 * usable.  0 makes every first wait give up at once: for tests of that path. */
int ismc_mlp_set_wait_limit(ismc_mlp* m, uint32_t polls);

/* ------------------------------------------------------------------------
 * Lookup-table inversion (Lookup/lookup.py:301-489).  Host arrays in and out
 * (row-major FP64); the table grid is R_i = i h, T_j = j h, h = 100/(N-1), in
 * percent, indexed [i][j].
 *   ismc_table_interp: linear interpolation of scattered samples (R, T, value)
 *     onto the table over the caller's triangulation tri[ntri][3] (Delaunay,
 *     as scipy.interpolate.griddata builds it, lookup.py:341-345); NaN outside.
 *   ismc_table_interp_cubic: the same table by Clough-Tocher cubic
 *     interpolation, the method griddata(method="cubic") applies in
 *     lookup.py:339-342.  nbr[ntri][3] holds the triangle across the edge
 *     opposite each vertex (-1 on the hull), as scipy.spatial.Delaunay's
 *     `neighbors`.  adj_ptr[npts+1] / adj is the vertex adjacency in CSR form
 *     (scipy's `vertex_neighbor_vertices`); pass NULL for both to derive it
 *     from the triangles.  Vertex gradients come from the global
 *     curvature-minimising estimate (Gauss-Seidel, tolerance 1e-6, at most
 *     400 sweeps) on the host; the per-cell cubic patches are evaluated on
 *     the GPU.
 *   ismc_table_uncertainty: lookup.py:349-376 -- per cell with finite,
 *     non-negative standard deviations, M normal draws of (R, T), nearest-cell
 *     values of both tables, 100 * std / value; NaN elsewhere.
 *   ismc_table_lookup: nearest cell of table_t[T_j][R_i] (the transposed table
 *     lookup.py returns) for n measurements (lookup.py:467-489).
 * ------------------------------------------------------------------------ */
int ismc_table_interp(const double* R, const double* T, const double* val, uint32_t npts,
                      const int32_t* tri, uint32_t ntri, uint32_t N, double* out);
int ismc_table_interp_cubic(const double* R, const double* T, const double* val, uint32_t npts,
                            const int32_t* tri, const int32_t* nbr, uint32_t ntri,
                            const int32_t* adj_ptr, const int32_t* adj, uint32_t N, double* out);
int ismc_table_uncertainty(const double* mua, const double* mus, const double* rstd,
                           const double* tstd, uint32_t N, uint32_t M, uint64_t seed,
                           double* mua_unc, double* mus_unc);
int ismc_table_lookup(const double* table_t, uint32_t N, const double* R, const double* T,
                      uint32_t n, double* out);

/* Sizes of the ABI structs, so bindings can check their own layouts. */
size_t ismc_sizeof(int which);   /* 0 stack, 1 spheres, 2 instance, 3 tally, 4 tune,
                                    5 solve_req, 6 solve_out */

#ifdef __cplusplus
}
#endif
#endif /* ISMC_GB300_H */
