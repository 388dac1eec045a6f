/*
 * Adjoint state shared by adjoint.cu (driver, DEM and fluid steps) and
 * adjoint_cpl.cu (the coupled SPH-DEM step).  Not part of the public ABI.
 */
#pragma once

#include <vector>

#include "internal.cuh"

namespace sphdem {

/* per-particle state record in tag order: r, v, vh, f, dens, dddt, fdrag
 * (the DEM drag the next middle phase spreads to the fluid), the pressure /
 * viscous force parts fp, fv of the fluid (read by the end phase's FPI),
 * and Omega of the end phase's continuity pass (VAR_H_CORRECTION) */
enum : int {
    AS_R = 0, AS_V = 3, AS_VH = 6, AS_F = 9, AS_DENS = 12, AS_DDDT = 13, AS_FDRAG = 14, AS_FP = 17, AS_FV = 20,
    AS_OME = 23, ADJ_NC = 24
};
constexpr int RM_NC = 4;           /* coupled: middle-phase record per particle, r and Omega of the force pass */
constexpr int ADJ_MAX_CONTACTS = 32;
constexpr int ADJ_AUX = 8;         /* SPH: r_s, vh_s, rho_s, pdr2_s */
constexpr int ADJ_NREC = 7;        /* SPH, mixed: float4 records per particle */
constexpr int SH_SHIFT = 26;       /* pair tables: partner tag bits below, image shift code above */
constexpr int ADJ_NGRAD = 5;       /* d/dk, d/dgamma, d/dalpha, d/dnu, d/d(drag scale) */
constexpr int CP_NACC = 24;        /* coupled step: accumulators per particle */
constexpr int CP_NEND = 15;        /* coupled step: end-phase results per particle */
constexpr int CP_NMID = 8;         /* coupled step: middle intermediates per particle */
constexpr int CP_NREC32 = 9;       /* coupled step, mixed: float4 records per particle */
constexpr int CP_FPI_PER = 384;    /* FPI partners per DEM particle per step (3D fluid at rest: ~122) */

/* one step's transposed pair table: (offset, count) per partner tag, the
 * owners' entries (owner tag | shift code of the owner's image) */
struct TrTable {
    int *nb = nullptr;
    int *ix = nullptr;      /* index of the pair's entry in the owners' table */
    int2 *oc = nullptr;
};
/* scratch of the transposition: counts, fill cursors, offsets, tile sums,
 * the entries before ranking */
struct TrScratch {
    int *cnt = nullptr, *fill = nullptr, *off = nullptr, *tsum = nullptr;
    int2 *tmp = nullptr;
};
constexpr int CP_NCOEF = 12;       /* coupled step: FPI coefficient record per DEM particle */

/* a grouped pair table of every step of a segment: entries partner tag |
 * shift << 26 grouped by particle, (offset, count) per tag and step, entries
 * used per step */
struct PairTable {
    int64_t cap = 0;                /* entries per step */
    int *nb = nullptr;
    int2 *oc = nullptr;
    int *cnt = nullptr;
    void alloc(int K, int64_t n);
    void free_all();
};

struct AdjointData {
    int mode = 0;
    int nsteps = 0, K = 0;
    /* tape store: nblk blocks of K step slots (K + 1 states) each; the
     * forward pass tapes the last nblk segments into blocks 0..nblk-1 */
    int nblk = 1;
    int blk = 0;                    /* block the current segment's tape is in */
    int taped = 0;                  /* the blocks hold the forward pass's tapes */
    int64_t n = 0;
    std::vector<double *> ckpt;     /* state at steps 0, K, 2K, ... and the final state */
    std::vector<DevGlobals> ckpt_g;
    double *seg = nullptr;          /* (K + 1) states of one segment */
    int4 *pairs = nullptr;          /* DEM: contacts of each step of a segment */
    int *pair_cnt = nullptr;        /* K counters (DEM contacts; SPH middle pairs) */
    double *adj = nullptr;          /* adjoint of the state (ADJ_NC per particle) */
    double *racc = nullptr;         /* accumulated adjoint of r1 through the forces */
    double *vmacc = nullptr;        /* DEM: adjoint of vhm; SPH: adjoint of vh1 */
    double *fbar = nullptr;         /* adjoint of f1 */
    double *mass = nullptr, *rad = nullptr;   /* tag order */
    int *typ = nullptr;             /* particle type, tag order */
    double *hh = nullptr;           /* smoothing length, tag order */
    /* SPH pair lists of each step of a segment: partner tag | shift code << 26,
     * grouped by particle; (offset, count) per tag */
    int64_t pair_cap = 0;           /* entries per step and list */
    int *nb_mid = nullptr, *nb_end = nullptr;
    int2 *oc_mid = nullptr, *oc_end = nullptr;
    int *cnt_end = nullptr;
    int *slot = nullptr;            /* step index inside the segment, read by the replay graph */
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    double *aux = nullptr;          /* SPH: r_s, vh_s, rho_s, pdr2_s per particle */
    float4 *rec = nullptr;          /* SPH, mixed: FP32 records, ADJ_NREC x n */
    double *grads = nullptr;        /* ADJ_NGRAD gradients */
    /* coupled step */
    PairTable cpl;                  /* fluid -> DEM pairs within Rc (middle phase), by fluid particle */
    PairTable fpi;                  /* DEM -> fluid pairs of calcFPI (end phase), by DEM particle */
    PairTable ct;                   /* DEM contacts (end phase), by DEM particle */
    int64_t ct_cap = 0;
    double *rmid = nullptr;         /* r and Omega after each step's middle phase, K x n x RM_NC */
    double *cacc = nullptr;         /* CP_NACC accumulators per particle */
    double *cend = nullptr;         /* CP_NEND end-phase results per particle */
    double *cmid = nullptr;         /* CP_NMID middle intermediates per particle */
    float4 *crec = nullptr;         /* mixed: CP_NREC32 FP32 records per particle */
    float4 *dpos = nullptr;         /* middle-phase DEM positions by state index (FP32) */
    int n_dem = 0;                  /* DEM particles at the forward pass */
    int *dem_tags = nullptr;        /* their tags */
    TapTables tap;                  /* mixed: the tables above as the forward coupling passes fill them */
    TrTable cplT, fpiT;             /* one step's coupling table by DEM particle, FPI table by fluid particle */
    TrScratch trw;
    double *coef = nullptr;         /* CP_NCOEF per particle (DEM): adjoints of its FPI sums */
    /* one step's pair geometry per entry of the coupling / FPI tables: (d,
     * W'/r) and W, FP32 on mixed handles, FP64 on FP64 handles */
    void *g4_cpl = nullptr, *gw_cpl = nullptr, *g4_fpi = nullptr, *gw_fpi = nullptr;
    double *hs = nullptr;           /* VAR_H_CORRECTION: the step's h_s per particle (tag order) */
};

/* G = (F(r, h_a) + F(r, h_b)) / 2 and dG/dr, F(r, h) = -10 C (2-q)^3 / h^(d+2)
 * (the Wendland C2 gradient factor of sph.h:322-342; 0 for q > 2) */
__device__ __forceinline__ void grad_factor(const DevCfg &c, double r, double ha, double hb, double &G, double &Gp) {
    G = 0.0;
    Gp = 0.0;
    const double hs[2] = {ha, hb};
    for (int k = 0; k < 2; k++) {
        const double h = hs[k], q = r / h;
        if (q > 2.0) continue;
        double ihn2 = 1.0 / (h * h);
        for (int d = 0; d < c.nd; d++) ihn2 /= h;
        const double t = 2.0 - q;
        G += -10.0 * c.wcon * (t * t * t) * ihn2;
        Gp += 30.0 * c.wcon * (t * t) * ihn2 / h;
    }
    G *= 0.5;
    Gp *= 0.5;
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* partner tag of a table entry and its image shift per axis */
__device__ __forceinline__ int table_entry(int e, int *sh) {
    const int code = (int)((unsigned)e >> SH_SHIFT);
    sh[0] = (code & 3) - 1;
    sh[1] = ((code >> 2) & 3) - 1;
    sh[2] = ((code >> 4) & 3) - 1;
    return e & ((1 << SH_SHIFT) - 1);
}

__device__ __forceinline__ int shift_code(const int *sh) {
    return ((sh[0] + 1) | ((sh[1] + 1) << 2) | ((sh[2] + 1) << 4)) << SH_SHIFT;
}

/* FP32 pair math of the mixed-precision reverse passes: Kahan sums, double-float
 * positions, and the gradient factor G, dG/dr */
struct Kf {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ void split2(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

template <int ND>
__device__ __forceinline__ float ipow_nd2(float ih) {   /* ih^(ND+2) */
    float v = ih * ih;
#pragma unroll
    for (int d = 0; d < ND; d++) v *= ih;
    return v;
}

/* G and dG/dr in FP32 (grad_factor) from 1/h of both particles */
template <int ND>
__device__ __forceinline__ void grad_factor32(float wcon, float r, float iha, float ihb, float &G, float &Gp) {
    G = 0.f;
    Gp = 0.f;
    const float ih[2] = {iha, ihb};
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float q = r * ih[k];
        if (q > 2.f) continue;
        const float t = 2.f - q, f = wcon * ipow_nd2<ND>(ih[k]);
        G += -10.f * f * (t * t * t);
        Gp += 30.f * f * (t * t) * ih[k];
    }
    G *= 0.5f;
    Gp *= 0.5f;
}

/* adjoint_cpl.cu: the coupled step */
void cpl_count_tables(sphdem_ctx *c, AdjointData *a);          /* sizes cpl / fpi / contacts (synchronises) */
void cpl_alloc(sphdem_ctx *c, AdjointData *a);
void cpl_free(AdjointData *a);
void cpl_reset_segment(sphdem_ctx *c, AdjointData *a);         /* empty tables before a segment's replay */
/* mixed handles: the forward coupling passes write the cpl / fpi / contact
 * tables while the replay graph is captured (c->tap = the returned tables) */
const TapTables *cpl_forward_taps(sphdem_ctx *c, AdjointData *a);
void cpl_taps_middle(sphdem_ctx *c, AdjointData *a);           /* inside the replay graph, after MIDDLE */
void cpl_taps_end(sphdem_ctx *c, AdjointData *a);              /* inside the replay graph, after END */
void cpl_backward_step(sphdem_ctx *c, AdjointData *a, int j, double dt);  /* VJP of step j of the segment */
bool cpl_overflow(sphdem_ctx *c, AdjointData *a);              /* a table of this segment overflowed (synchronises) */

}  // namespace sphdem
