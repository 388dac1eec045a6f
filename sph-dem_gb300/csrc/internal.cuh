/*
 * Host-side context of one handle and the launch entry points each .cu file
 * provides.  Not part of the public ABI (include/sphdem.h is).
 */
#pragma once

#include <string>
#include <vector>

#include "common.cuh"

struct sphdem_ctx;
namespace sphdem {
struct AdjointData;
}

namespace sphdem {

/* One timed launch (enabled by sphdem_kernel_times_reset(h, 1)). */
struct TimedLaunch {
    const char *name;
    cudaEvent_t ev0, ev1;
};

struct Buffers {
    int *skey = nullptr;     /* bucket key of each sorted particle        */
    int *perm = nullptr;     /* sorted slot -> previous slot              */
    int *slot = nullptr;     /* scatter scratch                           */
    int *slot_tag = nullptr;             /* tag and order key of the last-axis */
    unsigned long long *slot_z = nullptr; /* coordinate per scatter slot       */
    int *key = nullptr;      /* bucket key of each particle, previous order */
    int *cnt = nullptr;      /* bucket counts                             */
    int *start = nullptr;    /* bucket starts (exclusive scan)            */
    int *fill = nullptr;     /* scatter cursors                           */
    int *bsum = nullptr;     /* scan block sums                           */
    int *fields_d = nullptr; /* FP64 rows to gather at a rebuild          */
    int *fields_i = nullptr; /* int rows to gather                        */
    int n_fields_d = 0, n_fields_i = 0;
    int cells_cap = 0;       /* capacity of cnt/start/fill                */
    /* export scratch */
    int *pair_cnt = nullptr;
};

/* A per-step pair table in tag space that the mixed-precision forward
 * coupling passes fill while the adjoint's replay graph is captured: entries
 * partner tag | image shift code << 26, grouped by owner, at nb[slot * cap +
 * offset]; (offset, count) of each owner at oc[slot * n + tag]; cnt[slot]
 * counts the entries of the step (owners reserve with atomics), or exceeds
 * cap when the step's table overflowed.  `per` > 0: each owner has `per`
 * fixed slots (DEM-owned tables, owner w of the DEM range at w * per). */
struct TapTable {
    int *nb = nullptr;
    int2 *oc = nullptr;
    int *cnt = nullptr;
    int64_t cap = 0;
    int per = 0;
};
struct TapTables {
    TapTable cpl;   /* fluid -> DEM coupling pairs of the middle phase (porosity / drag passes) */
    TapTable fpi;   /* DEM -> fluid pairs of calcFPI (end phase) */
    TapTable ct;    /* DEM -> DEM contacts with positive overlap (end phase) */
    const int *slot = nullptr;   /* device step index inside the segment */
};

}  // namespace sphdem

struct sphdem_ctx {
    SphDemConfig host_cfg;
    sphdem::DevCfg cfg;
    int64_t n = 0, cap = 0;
    sphdem::DevState A, B;   /* B is the gather target of the next rebuild */
    bool flipped = false;    /* odd number of rebuilds so far              */
    sphdem::DevGlobals *g = nullptr;
    sphdem::Buffers buf;
    cudaStream_t stream = nullptr;
    std::string err;
    /* CUDA graphs of one full step, keyed by the state parity at its start
     * (bit 0) and whether the step re-initialises the density (bit 1), with
     * the parity each leaves behind */
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    bool graph_end_flip[4] = {false, false, false, false};
    long long host_step = 0;  /* host copy of the device step counter (sphStep) */
    /* CORRECTED_GRADIENT rows (CG_ROWS x cap) and the density re-initialisation's
     * first smoothing length (cap) */
    double *cg = nullptr, *hpred = nullptr;
    /* particles marked for deletion (state order), removed by the next rebuild */
    unsigned char *delmark = nullptr;
    long long population_gen = 0;   /* bumped by every insertion (captured graphs hold n) */
    bool in_capture = false;
    /* timing */
    bool timing = false;
    std::vector<sphdem::TimedLaunch> launches;
    std::vector<std::string> kt_names;
    std::vector<double> kt_ms;
    std::vector<long long> kt_count;
    /* mixed precision: packed FP32 particle records and neighbour lists */
    float4 *mx_pos = nullptr, *mx_vel = nullptr, *mx_aux = nullptr;
    int *mx_tg = nullptr;       /* type | ghost code << 8 */
    float *mx_om = nullptr;     /* Omega (VAR_H_CORRECTION) */
    int *mx_nbr = nullptr;      /* lists in tiles of 32 particles x 8 slots, mx_maxn x cap (rounded to 32) */
    int *mx_ncnt = nullptr;
    int mx_maxn = 0;
    bool mx_dem_only = false;   /* every particle at creation is DEM: the FP64 phases run */
    float4 *mx_q0 = nullptr, *mx_q1 = nullptr, *mx_q2 = nullptr;  /* FPI fields of fluid particles */
    float4 *mx_dp = nullptr;    /* (m/shep, fdrag) of DEM particles */
    float4 *mx_poslo = nullptr; /* low FP32 halves of offsets and h (double-float) */
    int4 *mx_rc4 = nullptr;     /* packed reference DEM buckets (own, image -L, image +L) */
    int4 *mx_win = nullptr;     /* coupling windows per SPH bucket index and axis */
    int mx_win_cap = 0;         /* entries per axis */
    float *mx_shep32 = nullptr; /* FP32 Shepard sums of DEM particles */
    float4 *mx_ds = nullptr;    /* DEM particles: offset in their SPH bucket, bucket key */
    float4 *mx_nb = nullptr;    /* boundary particles: FP32 normals n1 (+concave), n2, n3 */
    sphdem::AdjointData *adj = nullptr; /* checkpoints and buffers of the adjoint */
    /* device memory the adjoint may give its tape store (0: one segment's
     * tape; < 0: half of the free memory at the forward pass) */
    int64_t adj_tape_mem = 0;
    /* set while the adjoint's replay graph is captured: the mixed coupling
     * passes then also write these tables */
    const sphdem::TapTables *tap = nullptr;
    /* launch knobs chosen by the batch autotuner */
    int blk_pair = 128;         /* block size of the list-consumer passes (<= 128) */
    bool force_tile = false;    /* force / continuity: neighbour records staged in shared memory */
    int grid_div = 1;           /* divides the resident-block grid of the slice passes */
    int2 *mx_bandq = nullptr;   /* per particle: list entries within the FP32 band */
    int *mx_bandn = nullptr;    /* per particle: how many are recorded */
    int mx_band_per_particle = 0;
    sphdem::DevCfg *dcfg = nullptr;  /* device copy of cfg for out-of-line helpers */
    /* staging buffer for field transfers in tag order */
    double *stage = nullptr;
    /* asynchronous field transfers: two device staging buffers, the copy
     * stream, and per buffer the events of its gather and of its copy */
    cudaStream_t copy_stream = nullptr;
    double *astage[2] = {nullptr, nullptr};
    size_t astage_cap[2] = {0, 0};
    cudaEvent_t ev_gathered[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    bool astage_used[2] = {false, false};
    int acur = 0;
};

namespace sphdem {

/* CORRECTED_GRADIENT rows per particle: invM (nd x nd, row-major),
 * sumGrad/sum, sum */
enum : int { CG_M = 0, CG_C = 9, CG_S = 12, CG_ROWS = 13 };
inline bool corrected_gradient(const sphdem_ctx *c) { return c->host_cfg.flags & SPHDEM_F_CORRECTED_GRADIENT; }
inline bool reinit_configured(const SphDemConfig &c) { return c.reinit_dens_every > 0 || c.reinit_dens_at > 0; }
/* start() of step `step` re-initialises the density (sphIncompress.cpp:20) */
inline bool reinit_due(const SphDemConfig &c, long long step) {
    return (c.reinit_dens_every > 0 && step % c.reinit_dens_every == 0) ||
           (c.reinit_dens_at > 0 && step == c.reinit_dens_at);
}

/* launch bracket: records events around a launch when timing is enabled */
void launch_begin(sphdem_ctx *c, const char *name);
void launch_end(sphdem_ctx *c);

/* binning.cu */
void rebuild(sphdem_ctx *c);
void setup_rebuild_buffers(sphdem_ctx *c);

/* integrate.cu: elementwise phases and built-in hooks */
enum GlobalsOp { OP_MIDDLE_BEGIN = 0, OP_SET_DT, OP_END_BEGIN, OP_STEP_INC };
void globals_op(sphdem_ctx *c, int op);
void run_start(sphdem_ctx *c);
void run_hook_before_middle(sphdem_ctx *c);
void run_middle_tail(sphdem_ctx *c);
void run_end_drift(sphdem_ctx *c);
void run_end_tail(sphdem_ctx *c);
void run_hook_before_end(sphdem_ctx *c);
void run_hook_after_end(sphdem_ctx *c);
void run_h_derived(sphdem_ctx *c);

/* pairs64.cu / pairs32.cu: pair passes */
void run_porosity(sphdem_ctx *c);      /* calcPorosity + calcShepSum        */
void run_dem_drag(sphdem_ctx *c);      /* calcDEMtoSPHDrag + finalisePorosity */
void run_omega_eos(sphdem_ctx *c, bool omega, bool eos);
void run_force(sphdem_ctx *c);         /* calcForce + accelCondition        */
void run_dem_accel(sphdem_ctx *c);
void run_dddt(sphdem_ctx *c);          /* calcDddtDudt                      */
void run_invm(sphdem_ctx *c);
void run_dem_block(sphdem_ctx *c);     /* DEM_BLOCK: mean DEM force     */          /* calcInvM (CORRECTED_GRADIENT)     */
void run_reinit_density(sphdem_ctx *c); /* reset + ten rounds of calcHFromDens and calcDensity */
void run_dem_end(sphdem_ctx *c);       /* calcFPI + calcDEMContacts         */

void zero_dem_shep(sphdem_ctx *c);
void mixed_list_export(sphdem_ctx *c, int *cnt, const long long *offs, int *idx);

/* pairs32.cu: mixed-precision passes */
namespace mixed {
/* pack the FP32 records; `coupling` also packs the reference DEM buckets and
 * the coupling windows the SPH-DEM passes need */
void pack(sphdem_ctx *c, bool coupling = true);
void pack_fpi(sphdem_ctx *c);
void nlist(sphdem_ctx *c);
/* once per process, outside stream capture: kernel attributes of the step */
void prepare(sphdem_ctx *c);
void zero_shep(sphdem_ctx *c);
int nlist_max_count(sphdem_ctx *c);
int band_records_per_particle();
void omega_eos(sphdem_ctx *c, bool omega, bool eos);
void force(sphdem_ctx *c);
void dddt(sphdem_ctx *c);
void porosity(sphdem_ctx *c);
void dem_drag(sphdem_ctx *c);
void dem_end(sphdem_ctx *c);
}  // namespace mixed

/* pairs32.cu: the mixed lists of the last rebuild as the adjoint's pair
 * tables (tag space, slot *slot of nb / oc / cnt) */
void mixed_adj_pairs(sphdem_ctx *c, int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot);

/* population.cu: insertNewParticle / markForDeletion (synchronise) */
int insert_particles(sphdem_ctx *c, const SphDemParticles *in, int64_t *out_idx);
int mark_for_deletion(sphdem_ctx *c, const int64_t *idx, int64_t k);

/* diagnostics.cu: calcOutputVars on the device (synchronises) */
int output_vars(sphdem_ctx *c, SphDemOutputVars *out);

/* adjoint.cu */
void adjoint_free(sphdem_ctx *c);
constexpr int ADJ_MODE_DEM = 1;   /* all-DEM handle: contacts, walls, leapfrog */
constexpr int ADJ_MODE_SPH = 2;   /* fluid + fixed boundary particles, artificial viscosity */
constexpr int ADJ_MODE_COUPLED = 3;  /* fluid + fixed boundary + DEM, Morris viscosity, drag */
/* "" and the step family in *mode when the handle's step is covered, else why not */
std::string adjoint_supported(sphdem_ctx *c, int *mode);
int adjoint_forward(sphdem_ctx *c, int nsteps, int ckpt_every, int mode);
/* grads5 = d/d(dem_k), d/d(dem_gamma), d/d(alpha_artificial), d/d(viscosity),
 * d/d(drag_scale); *valid = the SPHDEM_GRAD_* bits the handle's step family
 * gives */
int adjoint_backward(sphdem_ctx *c, const double *seed_r, const double *seed_v, const double *seed_vh,
                     double *grads5, uint32_t *valid, double *dr0, double *dv0, double *dvh0);

/* capi.cu: one full step (all phases and hooks) on the handle's stream, one
 * phase of it, and the device error flags (synchronises) */
void step_sequence(sphdem_ctx *c);
void phase_sequence(sphdem_ctx *c, int phase);
int device_status(sphdem_ctx *c);

/* fields.cu */
struct FieldCopy {
    int row, ncomp;
    double *host;
};
/* gather the fields on the handle's stream, copy them on the copy stream;
 * returns without waiting */
void fields_get_async(sphdem_ctx *c, const FieldCopy *fc, int nf);
void fields_wait(sphdem_ctx *c);
void fields_async_free(sphdem_ctx *c);
void field_get(sphdem_ctx *c, int row, int ncomp, double *host);
void field_set(sphdem_ctx *c, int row, int ncomp, const double *host);
void field_get_int(sphdem_ctx *c, int row, int *host);

/* export.cu */
int export_pairs(sphdem_ctx *c, int kind, int64_t *offs, int32_t *idx, int64_t cap, int64_t *np);
int export_cells(sphdem_ctx *c, int32_t *cells);
int export_cells_noalloc(sphdem_ctx *c, int32_t *cells);

inline const DevState &cur(const sphdem_ctx *c) { return c->A; }

inline int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

}  // namespace sphdem

#define SPHDEM_CUDA_CHECK(expr)                                                  \
    do {                                                                         \
        cudaError_t e_ = (expr);                                                 \
        if (e_ != cudaSuccess)                                                   \
            throw std::string(#expr) + ": " + cudaGetErrorString(e_);            \
    } while (0)

#define SPHDEM_LAUNCH(ctx, name, kernel, grid, block, smem, ...)                \
    do {                                                                         \
        sphdem::launch_begin(ctx, name);                                         \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);         \
        sphdem::launch_end(ctx);                                                 \
    } while (0)
