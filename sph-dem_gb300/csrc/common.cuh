/*
 * Device-side types shared by every kernel of the SPH-DEM hot path.
 *
 * Layout in HBM (one handle):
 *   - particle state: structure of arrays, one contiguous FP64 block of
 *     NFD field rows x capacity (field-major, so a field row is one coalesced
 *     stream), plus NFI int32 rows.  Two copies (A/B): a rebuild sorts by
 *     bucket and gathers A -> B, then swaps.
 *   - bucket grids: one sorted particle order covers both grids -- every
 *     non-DEM particle first, sorted by SPH bucket, then DEM particles
 *     sorted by DEM bucket -- with one start[] array over all buckets.
 *   - DevGlobals: the step globals (time, dt, h_max, ghost widths, grid
 *     sizes, error flags) live in device memory so a whole step can be
 *     replayed as a CUDA graph without host round trips.
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sphdem.h"

namespace sphdem {

/* particle types (iamTypes, particle.h:17); DEAD marks a deleted particle */
enum : int {
    T_SPH = 0, T_SPHB = 1, T_BOUNDARY = 3, T_BOBJ1 = 5, T_BOBJ6 = 10,
    T_DEM = 11, T_DEMB = 12, T_IMMERSED = 13, T_DEAD = -1
};

__host__ __device__ inline bool is_sph_or_sphb(int t) { return t == T_SPH || t == T_SPHB; }
__host__ __device__ inline bool is_boundary(int t) { return t == T_BOUNDARY || (t >= T_BOBJ1 && t <= T_BOBJ6); }

/* ---- FP64 field rows ---- */
enum FieldD : int {
    FD_R = 0, FD_V = 3, FD_VHAT = 6, FD_V0 = 9, FD_VHAT0 = 12,
    FD_F = 15, FD_FP = 18, FD_FV = 21, FD_FB = 24,
    FD_FDRAG = 27, FD_FVEL = 30, FD_GPOR = 33,
    FD_N1 = 36, FD_N2 = 39, FD_N3 = 42,
    FD_MASS = 45, FD_DENS, FD_DDDT, FD_H, FD_PRESS, FD_PDR2, FD_OMEGA,
    FD_POR, FD_DPORDT, FD_SHEP, FD_RADIUS,
    FD_U, FD_DUDT, FD_EVISCF, FD_DEVISCF,   /* calcEnergies: elastic and viscous energy per unit mass, rates */
    FD_IH, FD_IHN, FD_IHN2,   /* 1/h, 1/h^nd, 1/h^(nd+2): refreshed whenever h changes */
    NFD
};
/* FI_RDC: reference DEM bucket (dem_getCellI) of DEM particles at the last rebuild */
enum FieldI : int { FI_IAM = 0, FI_TAG, FI_CONCAVE, FI_GCODE, FI_RDC0, FI_RDC1, FI_RDC2, NFI };

struct DevState {
    double *d;   /* NFD rows x cap */
    int *i;      /* NFI rows x cap */
    int64_t cap;
    __host__ __device__ __forceinline__ double *row(int f) const { return d + (int64_t)f * cap; }
    __host__ __device__ __forceinline__ int *irow(int f) const { return i + (int64_t)f * cap; }
};

/* Constant configuration (SphDemConfig plus derived numbers). */
struct DevCfg {
    int nd, visc, precision, n_walls;
    uint32_t flags;
    int periodic[3];
    double pi, rmin[3], rmax[3], dmin[3], dmax[3];
    double hfac, psep, h, dens, refd, gamma, prb, spsound, viscosity;
    double alpha_art, alpha_mon, bfac, maxdt, damptime;
    double dem_radius, dem_dens, dem_k, dem_gamma, dem_sr, dem_vol, rc;
    double dem_timestep, liq_dem_timestep, time_drop, freeze_until;
    double g_sph[3], g_dem[3];
    double wall_p[SPHDEM_MAX_WALLS][3], wall_n[SPHDEM_MAX_WALLS][3];
    double wcon;          /* WCON_WENDLAND for nd */
    double drag_scale;    /* factor on the Di Felice drag force */
    /* DEM search grid (static): cell size >= max(Rc, 2 DEM_SEARCH_RADIUS) */
    int ddims[3];
    double dcell[3], dorig[3], rdcell[3];
    /* migration test int((r-dmin)/dspace+1): extents and FP32 reciprocals */
    double dspace[3];
    float rdspace_f[3];
    /* DEM ghost test (width Rc): lower edge, span and FP32 reciprocal */
    double dg_lo[3], dg_sp[3];
    float dg_rsp_f[3];
    int n_dem_cells;
    int sph_cells_cap;    /* capacity of the SPH bucket grid */
    /* reference DEM bucket map (dem_getCellI) */
    double dem_cell_off;  /* 2*Rc/DSR - 1 */
    float rdem2_f;        /* 1/(2*DSR), FP32 */
    /* coupling search rule (dataLL.cpp:1154-1190) */
    int couple_num;       /* ceil(0.5*Rc/DSR) */
    double couple_lim;    /* (0.5*Rc/DSR)^2 */
    /* coupling kernel W(2r/Rc, Rc/2) constants */
    double two_over_rc, rc2, c_ihn, c_ihn2, c_hinv;
    double por_incr;      /* (4/3) PI DEM_RADIUS^3 [/(2 DEM_RADIUS) in 2D] */
    double k_anti;        /* K(1/HFAC) for anticlumping */
    /* FP32 copies for the mixed-precision boundary force */
    float f_pi, f_c0, f_rpsep, f_rdelp; /* PI, SPSOUND, 1/PSEP, 1/(BFAC*PSEP) */
    __host__ __device__ bool liq_dem() const { return flags & SPHDEM_F_LIQ_DEM; }
    __host__ __device__ bool var_h() const { return flags & SPHDEM_F_VAR_H_CORRECTION; }
};

/* Step globals and rebuild bookkeeping, resident in device memory. */
struct DevGlobals {
    double time, dt, new_dt, maxdt, dem_dt;
    double old_dt;                    /* dt of the previous step (middle() kick) */
    long long step;
    unsigned long long new_dt_bits;   /* atomicMin target (positive doubles) */
    double sr;                        /* sph_search_radius (dataLL.h:351) */
    double hmax;                      /* CdataLL::hmax */
    unsigned long long hmax_bits;     /* reduction target for the next hmax */
    double gw[27];                    /* procGhostMax2H per neighbour slot */
    unsigned long long slot_bits[27]; /* max ghost h per slot (reduction) */
    int sdims[3];                     /* SPH bucket grid extents */
    double scell[3];                  /* SPH bucket size per axis */
    double rscell[3];                 /* its reciprocal (periodic axes) */
    double sr2;                       /* 2*sph_search_radius */
    float rsr2_f;                     /* 1/(2*sph_search_radius), FP32 */
    /* SPH ghost test of the coming rebuild: lower edge, span, reciprocal */
    double ghost_lo[3], ghost_sp[3];
    float ghost_rsp_f[3];
    int n_sph_cells;
    int n_total_cells;                /* SPH + DEM buckets (+1 dead bucket) */
    int n_alive;
    long long n_deleted;
    double dem_avf[3];                /* DEM_BLOCK: mean DEM force of the end phase */
    unsigned int err;                 /* SPHDEM error bits (1 << code) */
    int err_info;
};

/* ---- exact FP64 helpers (no FMA contraction) ---- */
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

/* blitz dot for TinyVector: a0*b0 + (a1*b1 + a2*b2), computed exactly as the
 * reference does (no fused multiply-add). */
__device__ __forceinline__ double exact_len2(const double *d, int nd) {
    if (nd == 3) return dadd(dmul(d[0], d[0]), dadd(dmul(d[1], d[1]), dmul(d[2], d[2])));
    if (nd == 2) return dadd(dmul(d[0], d[0]), dmul(d[1], d[1]));
    return dmul(d[0], d[0]);
}

/* int((x - lo)/den + add), truncated toward zero, bit-identical to the
 * reference's FP64 expression.  An FP32 estimate decides unless the value
 * lies within its error bound of an integer; there the exact FP64 division
 * is taken.  (FP64 throughput is a small fraction of FP32 on this GPU, so
 * the exact path is kept for the rare ties.) */
__device__ __forceinline__ int trunc_index(double x, double lo, double den, float rden_f, double add) {
    const float q = ((float)x - (float)lo) * rden_f + (float)add;
    const float fl = floorf(q);
    const float margin = 1e-5f * (1.0f + fabsf(q)) + (fabsf((float)x) + fabsf((float)lo)) * 4e-7f * fabsf(rden_f);
    if (q - fl > margin && (fl + 1.0f) - q > margin && fabsf(q) < 1e6f)
        return q >= 0.0f ? (int)fl : (int)fl + 1;
    return (int)dadd(ddiv(dsub(x, lo), den), add);
}

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

/* atomic min / max of non-negative doubles through their bit patterns */
__device__ __forceinline__ void atomic_min_pos(unsigned long long *addr, double v) {
    if (v >= 0.0) atomicMin(addr, dbits(v));
}
__device__ __forceinline__ void atomic_max_pos(unsigned long long *addr, double v) {
    if (v >= 0.0) atomicMax(addr, dbits(v));
}

__device__ __forceinline__ void set_err(DevGlobals *g, int code, int info) {
    atomicOr(&g->err, 1u << code);
    g->err_info = info;
}

/* ---- sorted-order bucket decoding ---- */
struct CellCoord {
    int c[3];
};
__device__ __forceinline__ CellCoord decode_cell(int key, const int *dims, int nd) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    if (nd == 3) {
        cc.c[2] = key % dims[2];
        key /= dims[2];
        cc.c[1] = key % dims[1];
        cc.c[0] = key / dims[1];
    } else if (nd == 2) {
        cc.c[1] = key % dims[1];
        cc.c[0] = key / dims[1];
    } else {
        cc.c[0] = key;
    }
    return cc;
}

/* Neighbour bucket (self cell + offset) with periodic wrap.  Returns the
 * linear bucket or -1; shift[i] is -1/0/+1, the image the wrap stands for. */
__device__ __forceinline__ int neighbour_cell(const CellCoord &cc, int ox, int oy, int oz,
                                              const int *dims, const int *periodic, int nd,
                                              int shift[3]) {
    const int o[3] = {ox, oy, oz};
    int lin = 0;
    for (int i = 0; i < nd; i++) {
        int t = cc.c[i] + o[i];
        shift[i] = 0;
        if (t < 0) {
            if (!periodic[i]) return -1;
            t += dims[i];
            shift[i] = -1;
        } else if (t >= dims[i]) {
            if (!periodic[i]) return -1;
            t -= dims[i];
            shift[i] = 1;
        }
        lin = lin * dims[i] + t;
    }
    for (int i = nd; i < 3; i++) shift[i] = 0;
    return lin;
}

/* Ghost-image existence: the reference holds b's image shifted by `shift`
 * only if b lay within procGhostMax2H (or Rc for DEM) of the matching face
 * at the last rebuild (dataLL.cpp:522-582).  gcode packs, per axis, the
 * clipped inCoords (0, 1 or 2) in two bits. */
__device__ __forceinline__ bool image_exists(int gcode, const int shift[3], int nd) {
    for (int i = 0; i < nd; i++) {
        if (shift[i] == 0) continue;
        const int ic = (gcode >> (2 * i)) & 3;
        if (shift[i] < 0 ? ic != 2 : ic != 0) return false;
    }
    return true;
}

/* Image position component, exactly the reference's ghost shift formula
 * (RMIN-RMAX+r or RMAX-RMIN+r, dataLL.cpp:651-666). */
__device__ __forceinline__ double image_pos(double r, int shift, double rmin, double rmax) {
    if (shift == 0) return r;
    return shift > 0 ? dadd(dsub(rmax, rmin), r) : dadd(dsub(rmin, rmax), r);
}

/* reference DEM bucket index (dem_getCellI, dataLL.h:308-311) for one axis */
__device__ __forceinline__ int ref_dem_cell(double r, const DevCfg &c, int i) {
    return trunc_index(r, c.dmin[i], 2 * c.dem_sr, c.rdem2_f, c.dem_cell_off);
}

/* Does SPH particle s (reference DEM bucket cs) list DEM image d (bucket cd)
 * in calcNeighboursCoupling (dataLL.cpp:1154-1190)?  Returns 0 = bucket not
 * scanned, 1 = bucket added whole (addAll), 2 = added with r^2 < Rc^2. */
__device__ __forceinline__ int coupling_rule(const int *cs, const int *cd, const DevCfg &c) {
    int rP = 0, rM = 0;
    for (int i = 0; i < c.nd; i++) {
        const int o = cd[i] - cs[i];
        if (o < -c.couple_num || o > c.couple_num) return 0;
        rP += (o + 1) * (o + 1);
        rM += (o - 1) * (o - 1);
    }
    if (c.nd == 1) return 2;
    if (rP < c.couple_lim) return 1;
    if (rM < c.couple_lim) return 2;
    return 0;
}

/* bucket grid of the last rebuild as the pair passes read it, the bucket of
 * a position (SPH grid: getCellI, dataLL.h:303-305; DEM search grid), and
 * the 3^d stencil visit (x outer, z inner, as dataLL.cpp:1052-1071) */
struct GridInfo {
    int sdims[3];
    int n_sph_cells;
    double sr2, rscell[3];
    float rsr2_f;
};

__device__ __forceinline__ GridInfo load_grid(const DevGlobals *g) {
    GridInfo gi;
    for (int d = 0; d < 3; d++) {
        gi.sdims[d] = g->sdims[d];
        gi.rscell[d] = g->rscell[d];
    }
    gi.n_sph_cells = g->n_sph_cells;
    gi.sr2 = g->sr2;
    gi.rsr2_f = g->rsr2_f;
    return gi;
}

__device__ __forceinline__ CellCoord sph_cell_of(const DevCfg &c, const GridInfo &gi, const double *r) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    for (int d = 0; d < c.nd; d++) {
        int k;
        if (c.periodic[d]) {
            k = (int)floor((r[d] - c.dmin[d]) * gi.rscell[d]);
        } else {
            k = trunc_index(r[d], c.dmin[d], gi.sr2, gi.rsr2_f, 3.0);
        }
        if (k < 0) k = 0;
        if (k >= gi.sdims[d]) k = gi.sdims[d] - 1;
        cc.c[d] = k;
    }
    return cc;
}

__device__ __forceinline__ CellCoord dem_cell_of(const DevCfg &c, const double *r) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    for (int d = 0; d < c.nd; d++) {
        int k = (int)floor((r[d] - c.dorig[d]) * c.rdcell[d]);
        if (k < 0) k = c.periodic[d] ? c.ddims[d] - 1 : 0;
        if (k >= c.ddims[d]) k = c.periodic[d] ? 0 : c.ddims[d] - 1;
        cc.c[d] = k;
    }
    return cc;
}

/* visit every particle of the 3^d buckets around cc (x outer, z inner, as
 * dataLL.cpp:1052-1071) */
template <class Body>
__device__ __forceinline__ void scan_cells(const CellCoord &cc, const int *dims, const int *periodic, int nd,
                                           const int *start, int base, Body &&body) {
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (nd > 1 ? -1 : 0); oy <= (nd > 1 ? 1 : 0); oy++)
            for (int oz = (nd > 2 ? -1 : 0); oz <= (nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cc, ox, oy, oz, dims, periodic, nd, sh);
                if (lin < 0) continue;
                const int b0 = start[base + lin], b1 = start[base + lin + 1];
                for (int b = b0; b < b1; b++) body(b, sh);
            }
}

/* h = HFAC (m/rho)^(1/NDIM) (sphIncompress.h:698-700).  The FP64 path calls
 * pow like the reference; the mixed path takes an FP32 estimate of
 * x^(-1/NDIM) and one FP64 Newton step (relative error ~1e-14), because FP64
 * pow costs hundreds of FP64 operations on this GPU. */
__device__ __forceinline__ double smoothing_length(const DevCfg &c, double x) {
    if (c.precision != SPHDEM_PREC_MIXED) return c.hfac * pow(x, 1.0 / c.nd);
    if (c.nd == 1) return c.hfac * x;
    if (c.nd == 2) {
        double z = (double)rsqrtf((float)x);
        z = z * (1.5 - 0.5 * x * z * z);
        return c.hfac * x * z;
    }
    double z = (double)(1.0f / cbrtf((float)x));
    z = z * (4.0 - x * z * z * z) * (1.0 / 3.0);
    return c.hfac * x * z * z;
}

/* 1/h by an FP32 estimate and one FP64 Newton step in the mixed path */
__device__ __forceinline__ double recip(const DevCfg &c, double h) {
    if (c.precision != SPHDEM_PREC_MIXED) return 1.0 / h;
    double y = (double)(1.0f / (float)h);
    return y * (2.0 - h * y);
}

__device__ __forceinline__ void h_derived(const DevCfg &c, const DevState &s, int64_t i) {
    const double h = s.row(FD_H)[i];
    const double ih = recip(c, h);
    double ihn = ih;
    for (int d = 1; d < c.nd; d++) ihn *= ih;
    s.row(FD_IH)[i] = ih;
    s.row(FD_IHN)[i] = ihn;
    s.row(FD_IHN2)[i] = ihn * ih * ih;
}

}  // namespace sphdem
