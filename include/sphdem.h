/*
 * sphdem.h -- C ABI of the GB300-native SPH-DEM per-step particle hot path.
 *
 * One handle = one simulation resident in the HBM of one GPU; a batch
 * (sphdem_batch_*) steps an ensemble of independent handles together.  Every entry point returns an int status
 * (SPHDEM_OK == 0); no C++ exception crosses this boundary.  Text for the last
 * failure is available from sphdem_last_error().
 *
 * The functions replace the following interfaces of the reference
 * (martinjrobins/SPH-DEM, paths relative to the project root):
 *   - CdataLL constructor + reset()          dataLL.cpp:8-40, 140-236
 *   - CsphIncompress::start/middle/end       sphIncompress.cpp:3-38, 40-165, 167-251
 *   - the run loop and its hook sequence     run.cpp:102-119
 *   - the per-particle neighbour lists       dataLL.cpp:1026-1075 (calcNeighbours)
 *                                            dataLL.cpp:1104-1192 (calcNeighboursCoupling)
 *   - the bucket index maps                  dataLL.h:303-311 (getCellI, dem_getCellI)
 *   - the particle container (host AoS)      particle.h:62-316 (Cparticle), here SoA
 *
 * Threading contract: one handle per host thread.  All work of a handle is
 * ordered on that handle's private CUDA stream; calls returning data to the
 * host synchronise that stream.
 */
#ifndef SPHDEM_H
#define SPHDEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SPHDEM_OK                 0
#define SPHDEM_ERR_INVALID        1   /* bad argument or configuration            */
#define SPHDEM_ERR_CUDA           2   /* a CUDA runtime call failed               */
#define SPHDEM_ERR_CAPACITY       3   /* a fixed capacity (cells, pairs) exceeded  */
#define SPHDEM_ERR_OUT_OF_RANGE   4   /* a particle left the binning domain        */
#define SPHDEM_ERR_NOT_FINITE     5   /* NaN/Inf found in a state field            */
#define SPHDEM_ERR_UNSUPPORTED    6   /* option not built for this configuration   */
#define SPHDEM_ERR_TIMEOUT        7   /* a bounded device wait gave up             */

/* ---- particle types: values of iamTypes, particle.h:17 ------------------ */
#define SPHDEM_SPH            0
#define SPHDEM_SPH_BOUNDARY   1
#define SPHDEM_IMMOVABLE      2
#define SPHDEM_BOUNDARY       3
#define SPHDEM_GHOST          4
#define SPHDEM_DEM           11
#define SPHDEM_DEM_BOUNDARY  12
#define SPHDEM_IMMERSED_DEM  13

/* ---- viscosity models (customConstants.h #defines; sph.h:579-666) ------ */
#define SPHDEM_VISC_NONE        0
#define SPHDEM_VISC_ARTIFICIAL  1   /* VISC_ARTIFICIAL, sph.h:633-646      */
#define SPHDEM_VISC_MONAGHAN    2   /* VISC_MONAGHAN,   sph.h:606-630      */
#define SPHDEM_VISC_MORRIS      3   /* VISC_MORRIS,     sph.h:585-597      */

/* ---- feature flags (compile-time #defines of a case's customConstants.h) */
#define SPHDEM_F_CONST_H          (1u << 0)  /* CONST_H: h never updated        */
#define SPHDEM_F_NO_ANTICLUMPING  (1u << 1)  /* NO_ANTICLUMPING                 */
#define SPHDEM_F_VAR_H_CORRECTION (1u << 2)  /* VAR_H_CORRECTION (Omega terms)  */
#define SPHDEM_F_LIQ_DEM          (1u << 3)  /* LIQ_DEM: DEM + coupling         */
#define SPHDEM_F_FIXED_DT         (1u << 4)  /* dt == maxdt every step          */
#define SPHDEM_F_DEM_ONLY_CONTACT (1u << 5)  /* reserved                        */
#define SPHDEM_F_CORRECTED_GRADIENT (1u << 6) /* CORRECTED_GRADIENT (calcInvM, sph.h:394-434);
                                                 both precisions, no LIQ_DEM */
#define SPHDEM_F_DEM_BLOCK        (1u << 7)  /* DEM_BLOCK: every DEM particle takes the mean
                                                 DEM force before the end kick
                                                 (sphIncompress.cpp:231-238); needs LIQ_DEM */

/* ---- precision of the pair kernels ------------------------------------- */
#define SPHDEM_PREC_FP64   0   /* everything in FP64                                  */
#define SPHDEM_PREC_MIXED  1   /* FP32 pair math on FP64-cell-origin + FP32 offsets,
                                  Kahan-compensated FP32 sums, FP64 integration       */

/* A planar wall acting on DEM particles only: the device built-in form of a
 * case hook such as sediment3D/customSim.cpp:67-81 (addCustomBoundaries).
 * overlap = radius - dot(r - point, normal); force along +normal when > 0. */
typedef struct SphDemWall {
    double point[3];
    double normal[3];   /* unit, pointing into the domain */
} SphDemWall;

#define SPHDEM_MAX_WALLS 6

/* All case constants the reference takes from customConstants.h /
 * demConstants.h at compile time, passed at run time instead. */
typedef struct SphDemConfig {
    int32_t  ndim;                 /* NDIM: 1, 2 or 3 (the tests run 2 and 3)     */
    int32_t  visc_model;           /* SPHDEM_VISC_*                               */
    uint32_t flags;                /* SPHDEM_F_*                                  */
    int32_t  precision;            /* SPHDEM_PREC_*                               */
    int32_t  periodic[3];          /* PERIODIC[]                                  */
    int32_t  n_walls;              /* number of DEM walls used                    */
    double   pi;                   /* PI of the case (reference cases: 3.14159265)*/
    double   rmin[3], rmax[3];     /* RMIN[], RMAX[]: periodic extents            */
    double   domain_min[3];        /* globals.procDomain lower corner             */
    double   domain_max[3];        /* globals.procDomain upper corner             */
    double   hfac, psep, h;        /* HFAC, PSEP, H                               */
    double   dens, refd;           /* DENS, REFD                                  */
    double   gamma, prb, spsound;  /* GAMMA, PRB, SPSOUND                         */
    double   viscosity;            /* VISCOSITY (kinematic)                       */
    double   alpha_artificial;     /* ALPHA_ARTIFICIAL                            */
    double   bfac;                 /* BFAC (repulsive boundary)                   */
    double   maxdt;                /* globals.maxdt (== dt with SPHDEM_F_FIXED_DT) */
    double   damptime;             /* DAMPTIME                                    */
    double   dem_radius;           /* DEM_RADIUS (per-particle radius overrides)   */
    double   dem_dens;             /* DEM_DENS                                    */
    double   dem_k, dem_gamma;     /* DEM_K, DEM_GAMMA (LINEAR contact)            */
    double   dem_search_radius;    /* DEM_SEARCH_RADIUS                           */
    double   dem_vol;              /* DEM_VOL                                     */
    double   coupling_radius;      /* LIQ_DEM_COUPLING_RADIUS                     */
    double   dem_timestep;         /* DEM_TIMESTEP (demConstants.h:6)              */
    double   liq_dem_timestep;     /* LIQ_DEM_TIMESTEP (demConstants.h:19)         */
    double   time_drop_particle;   /* TIME_DROP_PARTICLE                          */
    double   freeze_dem_until;     /* built-in hook: DEM frozen while time <= this */
    double   gravity_sph[3];       /* built-in beforeMiddle hook, type sph only    */
    double   gravity_dem[3];       /* built-in beforeEnd hook, type dem only       */
    SphDemWall walls[SPHDEM_MAX_WALLS];
    double   drag_scale;           /* factor on the Di Felice drag force of calcParticleDrag
                                      (sph.h:1593-1598); 0 is read as 1, the reference's law */
    int32_t  reinit_dens_every;    /* REINIT_DENS_EVERY_N_STEPS: density re-initialisation of
                                      start() (sphIncompress.cpp:19-35) every that many steps;
                                      0 = never */
    int32_t  reinit_dens_at;       /* REINIT_DENS_AT_N_STEPS: and at that step (<= 0: never) */
} SphDemConfig;

/* Host-side particle arrays (structure of arrays).  Vector fields hold three
 * doubles per particle whatever ndim is (z unused in 2D).  Any pointer may be
 * NULL: that field is then not read (set) or not written (get).  Particles are
 * always presented in tag order (the order they were given to sphdem_create),
 * never in the device's cell-sorted order. */
typedef struct SphDemParticles {
    int64_t  n;
    int32_t *iam;          /* iamTypes                                           */
    int32_t *tag;
    uint8_t *concave;      /* boundary particle: concave corner flag              */
    double  *r, *v, *vhat; /* [3n]                                                */
    double  *mass, *dens, *h;
    double  *radius;       /* DEM radius; 0 or NULL -> cfg.dem_radius            */
    double  *norm1, *norm2, *norm3;  /* [3n] boundary normals                   */
    /* outputs (get only) */
    double  *f, *fp, *fv, *fb;       /* [3n]                                     */
    double  *dddt, *press, *pdr2;
    double  *porosity, *dporositydt, *shep_sum, *omega;
    double  *fdrag, *fvel, *grad_porosity;  /* [3n]                              */
    double  *v0, *vhat0;             /* [3n] start-of-step velocities            */
    /* calcEnergies integrals (sphIncompress.h:769-781), per unit mass: elastic
     * energy u and its rate, viscous energy eViscF and its rate (sph only) */
    double  *u, *dudt, *e_visc, *de_visc_dt;
} SphDemParticles;

/* Field-mask bits for get/set. */
#define SPHDEM_FIELD_R        (1u << 0)
#define SPHDEM_FIELD_V        (1u << 1)
#define SPHDEM_FIELD_VHAT     (1u << 2)
#define SPHDEM_FIELD_MASS     (1u << 3)
#define SPHDEM_FIELD_DENS     (1u << 4)
#define SPHDEM_FIELD_H        (1u << 5)
#define SPHDEM_FIELD_F        (1u << 6)   /* f, fp, fv, fb */
#define SPHDEM_FIELD_DDDT     (1u << 7)
#define SPHDEM_FIELD_PRESS    (1u << 8)   /* press, pdr2 */
#define SPHDEM_FIELD_COUPLING (1u << 9)   /* porosity, dporositydt, shep_sum, fdrag, fvel, grad_porosity */
#define SPHDEM_FIELD_OMEGA    (1u << 10)
#define SPHDEM_FIELD_V0       (1u << 11)  /* v0, vhat0 */
#define SPHDEM_FIELD_IAM      (1u << 12)
#define SPHDEM_FIELD_ENERGY   (1u << 13)  /* u, dudt, e_visc, de_visc_dt */
#define SPHDEM_FIELD_NORMALS  (1u << 14)  /* norm1, norm2, norm3 */
#define SPHDEM_FIELD_RADIUS   (1u << 15)
#define SPHDEM_FIELD_ALL      0xffffffffu

/* Step globals: the CglobalVars members of the hot path, globalVars.h:196-220. */
typedef struct SphDemGlobals {
    double  time, dt, new_dt, maxdt, dem_dt;
    int64_t sph_step;
    int64_t n_deleted;       /* particles removed for leaving the domain (dataLL.cpp:381-386) */
} SphDemGlobals;

/* Sizes of the current rebuild, for reporting and roofline arithmetic. */
typedef struct SphDemStats {
    int64_t n_particles, n_alive;
    int64_t n_list_pairs;    /* sum of the neighbour-list lengths (mixed precision) */
    int64_t list_depth;      /* allocated entries per particle                      */
    int64_t n_sph_cells, n_dem_cells;
    double  h_max, search_radius;
    int64_t n_band_candidates; /* pairs of the last list build decided in FP64 (mixed) */
    int64_t band_queue_capacity;
} SphDemStats;

/* Phases and built-in hook points, in the order run.cpp:112-118 calls them. */
#define SPHDEM_HOOK_BEFORE_START   0
#define SPHDEM_PHASE_START         1
#define SPHDEM_HOOK_BEFORE_MIDDLE  2
#define SPHDEM_PHASE_MIDDLE        3
#define SPHDEM_HOOK_BEFORE_END     4
#define SPHDEM_PHASE_END           5
#define SPHDEM_HOOK_AFTER_END      6

/* Pair lists exported for parity checks. */
#define SPHDEM_PAIRS_SPH        0  /* calcNeighbours for non-DEM particles       */
#define SPHDEM_PAIRS_DEM        1  /* calcNeighbours for DEM particles           */
#define SPHDEM_PAIRS_COUPLE_SD  2  /* calcNeighboursCoupling, SPH -> DEM, r < Rc   */
#define SPHDEM_PAIRS_COUPLE_DS  3  /* calcNeighboursCoupling, DEM -> SPH          */

typedef struct sphdem_ctx *sphdem_handle;

/* Create a simulation from host particles.  Replaces `new CdataLL(ps,globals,
 * true)` (run.cpp:80, dataLL.cpp:8-40): copies the particles to HBM, sizes the
 * bucket grids and performs the first rebuild.  `capacity` is the maximum
 * particle count the handle will ever hold (>= init->n). */
int sphdem_create(const SphDemConfig *cfg, const SphDemParticles *init,
                  int64_t capacity, sphdem_handle *out);
/* Release the handle's device memory (the reference's particle container and
 * CdataLL live until the process ends, run.cpp:163-164). */
int sphdem_destroy(sphdem_handle h);

/* Run one phase or built-in hook point (SPHDEM_PHASE_* / SPHDEM_HOOK_*).
 * PHASE_START/MIDDLE/END replace CsphIncompress::start/middle/end
 * (sphIncompress.cpp:3-251); the HOOK_* points apply the built-in hooks of the
 * configuration (gravity, DEM walls, DEM freeze) that a case's customSim
 * would apply at that point.  A host-side hook instead uses get/set_fields. */
int sphdem_phase(sphdem_handle h, int phase);

/* nsteps full steps of the run loop (run.cpp:102-118): sph_step++, then the
 * seven phases/hooks in run.cpp order.  Consecutive calls replay one captured
 * CUDA graph of a step. */
int sphdem_step(sphdem_handle h, int nsteps);

/* Read / write the fields `mask` selects, in tag order: what hook and output
 * code reads and writes on the reference's particle container
 * (data->getParticles(), dataLL.h:237-238; the Cparticle members,
 * particle.h:262-316).  set_fields writes r, v, vhat, f (f, fp, fv, fb),
 * dens, h, normals, radius, coupling, energy and dddt groups. */
int sphdem_get_fields(sphdem_handle h, uint32_t mask, SphDemParticles *out);
int sphdem_set_fields(sphdem_handle h, uint32_t mask, const SphDemParticles *in);
/* sphdem_get_fields without waiting (no counterpart in the reference, whose
 * particles live in host memory): the fields are gathered into tag order on
 * the handle's stream and copied into `out` on a separate copy stream, so the
 * copy overlaps the steps that follow.  `out`'s arrays must stay valid and
 * unread until sphdem_fields_wait returns; pinned host memory
 * (sphdem_alloc_host) makes the copy truly asynchronous.  Two transfers
 * overlap; a third waits on the device for the first to finish.  Integer
 * fields (iam, tag) are not copied by this call. */
int sphdem_get_fields_async(sphdem_handle h, uint32_t mask, const SphDemParticles *out);
/* Wait for the handle's sphdem_get_fields_async copies (no counterpart). */
int sphdem_fields_wait(sphdem_handle h);
/* The step globals of CglobalVars (globalVars.h:196-220): time, dt, new dt,
 * maxdt, DEM dt, sphStep; set_globals writes time, dt, maxdt and sphStep. */
int sphdem_get_globals(sphdem_handle h, SphDemGlobals *out);
/* Sizes of the current rebuild (no counterpart; for reporting). */
int sphdem_get_stats(sphdem_handle h, SphDemStats *out);
int sphdem_set_globals(sphdem_handle h, const SphDemGlobals *in);

/* Insert in->n particles between phases (CdataLL::insertNewParticle,
 * dataLL.cpp:238-261, called from a case hook).  iam, r, mass, dens and h
 * are required; v, vhat (default v), radius, normals and concave are read if
 * given, every other field starts as sphdem_create leaves it.  Each new
 * particle takes the lowest free tag-order index -- a slot left by a deleted
 * particle, else the next index past the last -- written to out_idx[j] when
 * out_idx is not NULL.  Past the capacity given at creation nothing is
 * inserted and the call returns SPHDEM_ERR_CAPACITY (the reference exits at
 * MAX_NUM_PARTICLES_PER_CPU).  The new particles join the bucket lists at the
 * next rebuild, which every phase's neighbour passes follow. */
int sphdem_insert_particles(sphdem_handle h, const SphDemParticles *in, int64_t *out_idx);

/* Mark particles (tag-order indices) for deletion (CdataLL::markForDeletion,
 * dataLL.cpp:263-266: tag = -111).  They take part in the step as usual
 * until the next rebuild removes them (dataLL.cpp:377-380); their slots are
 * then free for insertion.  An index out of range or of a deleted particle
 * gives SPHDEM_ERR_INVALID and marks nothing. */
int sphdem_mark_for_deletion(sphdem_handle h, const int64_t *idx, int64_t k);

/* Rebuild the bucket lists at the current positions (CdataLL::reset,
 * dataLL.cpp:140-236): periodic wrap, out-of-domain deletion, h_max tracking,
 * bin, sort by cell, permute. */
int sphdem_rebuild(sphdem_handle h);

/* Export one neighbour relation as CSR over tag order: calcNeighbours
 * (dataLL.cpp:1026-1075) for SPHDEM_PAIRS_SPH / _DEM, calcNeighboursCoupling
 * (dataLL.cpp:1104-1192) for the two coupling directions.  `offsets` has n+1
 * entries, `idx` holds neighbour tags' positions (tag order index).  Pass
 * idx == NULL to query the pair count in *n_pairs. */
int sphdem_pairs(sphdem_handle h, int kind, int64_t *offsets, int32_t *idx,
                 int64_t idx_capacity, int64_t *n_pairs);

/* Output-step diagnostics: the globals CsphIncompress::calcOutputVars
 * (sphIncompress.h:274-319) computes at each output step of run.cpp:131 --
 * momenta and energies of the sph particles, maxima, mean and variance of the
 * density over sph and sphBoundary particles, the rms difference between the
 * density and its SPH summation (calcAveDensFromMass, 266-272).  n counts all
 * live particles, as the reference's particle container does; ff, eViscB and
 * eBForce are zero on the reference's path as well (never accumulated). */
typedef struct SphDemOutputVars {
    double  lin_mom[3], ang_mom;
    double  e_ke, e_elast, e_elast_exact, ed_elast_dt;
    double  e_visc_f, ed_visc_f_dt, e_ff, ed_ff_dt, e_visc_b, e_b_force, e_total;
    double  max_v, max_f, max_ff, rms_ff;
    double  ave_dens, var_dens, ave_dens_from_mass;
    int64_t n, n_sph;
} SphDemOutputVars;

/* CsphIncompress::calcOutputVars (sphIncompress.h:274-319) on the device */
int sphdem_output_vars(sphdem_handle h, SphDemOutputVars *out);

/* Bucket index of every particle (tag order) in the reference's own maps:
 * getCellI (dataLL.h:303-305) for non-DEM, dem_getCellI (dataLL.h:308-311)
 * for DEM, as int32 triples (unused z = 0). */
int sphdem_cell_ids(sphdem_handle h, int32_t *cell_xyz);

/* ---------------------------------------------------------------------- */
/* Adjoint (reverse-mode gradients) of the step: no counterpart in the
 * reference, which has no derivatives.  Covers, with fixed dt and no
 * damping:
 *  - handles whose particles are all DEM (LIQ_DEM without fluid, no
 *    freezing; at most 67,108,863 particles): gradients dem_k, dem_gamma
 *    and the initial state;
 *  - fluid handles of SPH and SPH-boundary particles (no LIQ_DEM) with
 *    artificial viscosity, CONST_H, NO_ANTICLUMPING, no VAR_H_CORRECTION and
 *    no periodic axes (the dam break; at most 4M particles): gradients
 *    `viscosity` = dL/d(alpha_artificial) and the initial state;
 *  - coupled LIQ_DEM handles of SPH, SPH-boundary and DEM particles with
 *    Morris viscosity, NO_ANTICLUMPING, gamma = 7 and either CONST_H or, on
 *    mixed-precision handles, VAR_H_CORRECTION with h following the density
 *    (periodic axes allowed; sedimentation; at most 4M particles):
 *    gradients dem_k, dem_gamma, `viscosity` = dL/d(kinematic viscosity),
 *    drag_scale and the initial state.
 * Other handles get SPHDEM_ERR_UNSUPPORTED.
 *
 * sphdem_adjoint_forward runs nsteps ordinary steps from the current state,
 * keeping a device checkpoint every ckpt_every steps.
 * sphdem_adjoint_backward takes the adjoint of the final r, v and vhat (tag
 * order, 3 per particle; NULL = zero), replays each checkpoint segment once
 * and applies the step's vector-Jacobian product in reverse order.  It
 * returns the gradients flagged in grads->valid and the adjoints of the
 * initial r, v and vhat (NULL to skip), and leaves the handle at the final
 * state.  SPHDEM_ERR_CAPACITY: a step used more pairs than the lists sized
 * at the forward pass hold. */
#define SPHDEM_GRAD_DEM_K      (1u << 0)
#define SPHDEM_GRAD_DEM_GAMMA  (1u << 1)
#define SPHDEM_GRAD_POSITIONS  (1u << 2)
#define SPHDEM_GRAD_VISCOSITY  (1u << 3)
#define SPHDEM_GRAD_DRAG_SCALE (1u << 4)

typedef struct SphDemGrads {
    double dem_k, dem_gamma, viscosity, drag_scale;
    uint32_t valid;             /* SPHDEM_GRAD_* bits of the entries computed */
} SphDemGrads;

/* Adjoint forward pass (no counterpart in the reference, see above). */
int sphdem_adjoint_forward(sphdem_handle h, int nsteps, int ckpt_every);
/* Device memory the adjoint may use to keep checkpoint segments' tapes (the
 * per-step states and pair tables the reverse sweep reads) from the forward
 * pass: bytes = 0 (the default) keeps one segment's tape, so the backward
 * pass replays every earlier segment from its checkpoint; bytes > 0 keeps
 * the tapes of as many of the last segments as fit, which the backward pass
 * then does not replay; bytes < 0 takes half of the device memory free at
 * sphdem_adjoint_forward.  Applies from the next sphdem_adjoint_forward.
 * All-DEM handles always keep one segment's tape. */
int sphdem_adjoint_set_tape_memory(sphdem_handle h, int64_t bytes);
/* Adjoint backward pass (no counterpart in the reference, see above). */
int sphdem_adjoint_backward(sphdem_handle h, const double *dL_dr, const double *dL_dv,
                            const double *dL_dvhat, SphDemGrads *grads,
                            double *dL_dr0, double *dL_dv0, double *dL_dvhat0);

/* ---------------------------------------------------------------------- */
/* Batched ensembles: no counterpart in the reference, which runs one
 * simulation per process.  A batch steps many independent handles (any
 * particle counts, configurations and time steps) with one CUDA graph per
 * step whose branches are the members' own step sequences.  Members stay
 * usable on their own (get/set fields, stats); a batch call orders itself
 * after their pending work and their later calls after it.  Destroy the
 * batch before its members.  A member with a density re-initialisation
 * (reinit_dens_every / reinit_dens_at) gives SPHDEM_ERR_UNSUPPORTED. */
typedef struct sphdem_batch_ctx *sphdem_batch;

/* Batches have no counterpart in the reference, which runs one simulation
 * per process (run.cpp:16-164). */
int sphdem_batch_create(const sphdem_handle *members, int n, sphdem_batch *out);
int sphdem_batch_destroy(sphdem_batch b);
/* nsteps full steps of every member (hooks on the device, as sphdem_step) */
int sphdem_batch_step(sphdem_batch b, int nsteps);
/* one untimed step, then device time of nsteps graph replays in *ms */
int sphdem_batch_time_steps(sphdem_batch b, int nsteps, double *ms);
/* Autotuner: for every member, times steps_per_trial graph-replayed steps
 * alone for each candidate launch configuration (block size of the
 * list-consumer passes 64 / 128, grid of the slice passes full or 1/4,
 * neighbour tiles of the force and continuity passes staged in shared
 * memory or read through L1 -- mixed 2D / 3D handles) and keeps the
 * fastest.  Choices are remembered per (dimension, precision, feature
 * flags, particle-count octave) for the process: a member of a class tuned
 * before takes its choice untimed.  A timed member advances by up to
 * 8 x (steps_per_trial + 1) steps.  `chosen` (optional, 3 ints per member)
 * receives block size, grid divisor and staged tiles (0 / 1). */
int sphdem_batch_tune(sphdem_batch b, int steps_per_trial, int *chosen);
/* Text of b's last failure; with b == NULL, of the calling thread's last
 * failed sphdem_batch_create ("no batch" if there was none). */
int sphdem_batch_last_error(sphdem_batch b, char *buf, size_t len);

/* Largest particle count sphdem_cell_ids_noalloc accepts. */
#define SPHDEM_CELL_IDS_NOALLOC_MAX 262144

/* sphdem_cell_ids without any device allocation: no counterpart in the
 * reference (whose cell indices are host arrays).  For callers that must not
 * allocate device memory, e.g. a diagnostics hook after an out-of-memory
 * failure, or a loop that cannot take the device-wide synchronisation of
 * cudaFree.  It stages through one static device array of
 * SPHDEM_CELL_IDS_NOALLOC_MAX x 3 int32 per device, shared by every call on
 * that device: calls that overlap in time race on it.  Larger simulations
 * return SPHDEM_ERR_CAPACITY.  Every call looks the array's address up on the
 * handle's device; the first call on a device may load the module there, so
 * make it before any stream capture on that device.  Same output as
 * sphdem_cell_ids. */
int sphdem_cell_ids_noalloc(sphdem_handle h, int32_t *cell_xyz);

/* Per-kernel device time accumulated with CUDA events since the last reset
 * (names separated by '\n' in `names`, times in ms, launch counts).  No
 * counterpart: the reference times whole phases with gettimeofday
 * (run.cpp:96-100, globalVars.h:163-188). */
int sphdem_kernel_times(sphdem_handle h, char *names, size_t names_len,
                        double *ms, int64_t *launches, int max_kernels,
                        int *n_kernels);
int sphdem_kernel_times_reset(sphdem_handle h, int enable);

/* Time `nsteps` full steps on the handle's stream with CUDA events (no
 * counterpart). */
int sphdem_time_steps(sphdem_handle h, int nsteps, double *ms);

/* Page-locked host buffers for get/set_fields: transfers from and to them run
 * at full link bandwidth.  (No counterpart in the reference, which has no
 * device; a convenience for callers that stream fields every step.) */
int sphdem_alloc_host(size_t bytes, void **ptr);
int sphdem_free_host(void *ptr);

/* Text of h's last failure; with h == NULL, of the calling thread's last
 * failed sphdem_create ("no handle" if there was none).  The reference
 * prints to cerr and exits instead (dataLL.cpp:207-211). */
int sphdem_last_error(sphdem_handle h, char *buf, size_t len);
const char *sphdem_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SPHDEM_H */
