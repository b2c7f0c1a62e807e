// ismc_dev.h -- device-side data layout of the propagator (shared by the
// kernels and the host library; not part of the public ABI).
#pragma once
#include <stdint.h>
#include "../../include/ismc.h"

#define ISMC_HDR_WORDS 44
#define ISMC_LAYER_FIELDS 16

// Layer flags
#define ISMC_LF_GLASS 1u   // mus == 0: no scattering (ISMLMC.py:81, MLMC.py:97)
#define ISMC_LF_ISO   2u   // g == 0: isotropic phase function (MLMC.py:183)

// Instance flags
#define ISMC_IF_RSPHERE 1u
#define ISMC_IF_TSPHERE 2u

// Per-layer constants, grouped so that each event reads them as 16-byte
// shared-memory words: q0 what an interaction needs, q1 the Henyey-Greenstein
// constants, q2 the geometry and interface index ratios, q3 the rest.
struct DevLayer {
    float mut, inv_mut, drop, hgc;          // q0; drop: tissue mua/mut per interaction, glass mua (1/cm)
    float hgd, hge, hga, hgb;               // q1: 1-g, 2g, 1/(2g), 1+g^2 (hgc = 1-g^2)
    float z_top, z_bot, eta_up, eta_dn;     // q2: eta_up = n/n(above), eta_dn = n/n(below)
    float n;                                // q3
    uint32_t lflags;
    uint32_t _pad[2];
};
static_assert(sizeof(DevLayer) == 64, "DevLayer layout");

// Prepared instance: everything the walk needs, derived once per launch by
// ismc_prepare_kernel: a 44-word header, then one DevLayer per layer.  One
// warp copies it word by word into its shared-memory slot.
struct DevInst {
    // header: 40 words
    uint32_t L, mode, flags, stream;
    uint32_t seed_lo, seed_hi;
    float t_tot;                // total thickness (bottom of the stack)
    float cos_port[2];          // |mu_z| >= cos_port -> specular (R) / unscattered (T)
    float p_reinc[2];           // sphere re-incidence probability (sphere multiplier)
    float ux0, uz0;             // launch direction
    float roul_thr, roul_m, roul_inv_m;
    float eta_in[2];            // 1/n of the top / bottom layer (ambient -> sample)
    uint32_t stream_k1;         // stream ^ rk[1]: the constant half of Philox round 0
    uint32_t _hpad;
    // Philox key schedule of the instance's seed: round r uses
    // (rk[2r], rk[2r+1]) = (seed_lo + r W0, seed_hi + r W1) mod 2^32, read as
    // five 16-byte words (byte offset 80, 16-byte aligned)
    uint32_t rk[20];
    // the launch's incidence, the same for every packet of the instance: the
    // reflection probability and refracted cosine the incidence event would
    // compute for the launch direction (same operations, so the same bits)
    float launch_R, launch_ct;
    uint32_t _hpad2[2];
    DevLayer ly[ISMC_MAXL];     // per-layer constants, 64 B each
};

static_assert(sizeof(DevInst) == 4 * (ISMC_HDR_WORDS + ISMC_LAYER_FIELDS * ISMC_MAXL),
              "DevInst layout");

// Packet range of an instance (the queue decodes chunks from these).
struct DevRange {
    uint64_t offset;            // first packet id
    uint64_t count;             // packets
};

// Tally block in device memory: same layout as ismc_tally so it can be copied
// back verbatim.  Counters are added with 64-bit integer atomics.
static_assert(sizeof(ismc_tally) == 8 * 16 + 4 * 4, "ismc_tally layout");

struct PropParams {
    const DevInst* inst;
    const DevRange* range;
    const unsigned long long* chunk_prefix;   // n_inst + 1 entries
    ismc_tally* tally;
    unsigned long long* ctrl;                 // [0] queue head, [1] packets per chunk
    uint32_t n_inst;
    uint32_t max_events;
};

// Host-callable launchers (defined in ismc_kernels.cu).
//   chunk_override: packets per queue chunk, 0 = derive on the device from the
//   batch's total packets so that every warp gets ~chunks_per_warp chunks.
extern "C++" {
int ismc_launch_prepare(const ismc_instance* d_in, uint32_t n_inst, DevInst* d_inst,
                        DevRange* d_range, unsigned long long* d_prefix, ismc_tally* d_out,
                        unsigned long long* d_ctrl, uint32_t chunk_override, uint32_t total_warps,
                        uint32_t chunks_per_warp, void* stream);
int ismc_launch_propagate(const PropParams& p, uint32_t blocks, uint32_t threads, void* stream);
int ismc_propagate_occupancy(uint32_t threads, int* blocks_per_sm);
// Record a library-level error (no context): text for ismc_last_error(NULL).
int ismc_lib_error(int code, const char* fmt, ...);
}
