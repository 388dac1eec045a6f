/*
 * Mixed-precision pair passes (SPHDEM_PREC_MIXED).
 *
 * Positions stay FP64 in the state; for the pair math every particle is
 * packed, once per rebuild, as an FP32 offset from the FP64 origin of its own
 * bucket plus FP32 h / velocity / mass / density / pdr2.  The displacement of
 * a pair in buckets ca and cb = ca + o is (off_a - off_b) - o*bucket, all FP32
 * and well conditioned (|off| < one bucket).  Every kernel is specialised on
 * the dimension so per-axis arrays live in registers.
 *
 *   k_nlist      after each rebuild, the exact neighbour list of every
 *                sph/sphBoundary particle: one warp per SPH bucket stages the
 *                3^d stencil's candidates in shared memory and tests them in
 *                FP32 with a proven error bound; candidates inside the bound
 *                go to k_band_fix (double-float, then the reference's FP64
 *                predicate, particle.h:236-238, for true ties).  Periodic
 *                images only where the reference holds a ghost.  Entries
 *                b | stencil code << 26 in tiles of 32 particles x 8 slots
 *                (nl_at).
 *   k_omega_eos  calcOmega over the list + the FP64 EOS (its (rho/rho0)^7-1
 *                cancels too much for FP32)
 *   k_force      calcForce + the Courant/viscous/accel dt conditions
 *   k_dddt       calcDddtDudt
 *   k_couple     calcPorosity + calcShepSum (mode 0) and calcDEMtoSPHDrag +
 *                finalisePorosity (mode 1): 32-particle slices stage the DEM
 *                particles of the DEM buckets within Rc in shared memory and
 *                test them with the reference's asymmetric bucket rule
 *                (dataLL.cpp:1154-1190); the Shepard scatter is reduced over
 *                the warp and lands as one FP64 atomic per (warp, DEM particle)
 *   k_dem_end    calcFPI + calcParticleDrag + calcDEMContacts: one warp per
 *                DEM particle, lanes split the candidates, warp reductions
 *
 * Sums are Kahan-compensated in FP32 and added to the FP64 state once per
 * particle.  Roofline: the list passes are FP32-pipe-bound on 3D workloads
 * (~80 FP32 FLOP per listed pair against 4 B of list + 48 B of packed input).
 */
#include <algorithm>
#include <cfloat>
#include <climits>
#include <vector>

#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 128;
constexpr int B_BITS = 26;
constexpr int B_MASK = (1 << B_BITS) - 1;

struct Kahan {
    float s, c;
    __device__ __forceinline__ void init(float v) {
        s = v;
        c = 0.f;
    }
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

/* A plain FP32 sum with the same interface, for sums whose rounding does
 * not reach the results' tolerance: the calcOmega sum under
 * VAR_H_CORRECTION, where Omega = 1 + h sum / (rho NDIM) is an O(1) factor
 * known to ~1e-6 from ~100 terms. */
struct Plain {
    float s;
    __device__ __forceinline__ void init(float v) { s = v; }
    __device__ __forceinline__ void add(float x) { s += x; }
};

__device__ __forceinline__ float wK32(float q, float wcon) {
    if (q > 2.f) return 0.f;
    const float t = 2.f - q, t2 = t * t;
    return wcon * (t2 * t2) * (1.f + 2.f * q);
}
__device__ __forceinline__ float wdK32(float q, float wcon) {
    if (q > 2.f) return 0.f;
    const float t = 2.f - q, t2 = t * t;
    return wcon * (-4.f * (t2 * t) * (1.f + 2.f * q) + 2.f * (t2 * t2));
}

/* error-free transforms for the double-float (hi + lo FP32) refinement */
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = a * b;
    e = fmaf(a, b, -p);
}

template <int ND>
__device__ __forceinline__ float powi(float x) {
    float r = x;
#pragma unroll
    for (int k = 1; k < ND; k++) r *= x;
    return r;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* FP64 origin of SPH bucket `cell` on axis d, and its size */
__device__ __forceinline__ double sph_origin(const DevCfg &c, const DevGlobals *g, int d, int cell) {
    return c.periodic[d] ? c.dmin[d] + cell * g->scell[d] : c.dmin[d] + (cell - 3) * g->sr2;
}
__device__ __forceinline__ double sph_width(const DevCfg &c, const DevGlobals *g, int d) {
    return c.periodic[d] ? g->scell[d] : g->sr2;
}
__device__ __forceinline__ double dem_origin(const DevCfg &c, int d, int cell) {
    return c.dorig[d] + cell * c.dcell[d];
}

template <int ND>
__device__ __forceinline__ void decode(int key, const int *dims, int *cc) {
    if (ND == 3) {
        cc[2] = key % dims[2];
        key /= dims[2];
        cc[1] = key % dims[1];
        cc[0] = key / dims[1];
    } else if (ND == 2) {
        cc[1] = key % dims[1];
        cc[0] = key / dims[1];
    } else {
        cc[0] = key;
    }
}

/* stencil neighbour (offsets o) with periodic wrap; -1 when off the grid */
template <int ND>
__device__ __forceinline__ int nb_cell(const int *cc, const int *o, const int *dims, const int *periodic, int *sh) {
    int lin = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        int t = cc[d] + o[d];
        sh[d] = 0;
        if (t < 0) {
            if (!periodic[d]) return -1;
            t += dims[d];
            sh[d] = -1;
        } else if (t >= dims[d]) {
            if (!periodic[d]) return -1;
            t -= dims[d];
            sh[d] = 1;
        }
        lin = lin * dims[d] + t;
    }
    return lin;
}

template <int ND>
__device__ __forceinline__ bool img_ok(int gcode, const int *sh) {
#pragma unroll
    for (int d = 0; d < ND; d++) {
        if (sh[d] == 0) continue;
        const int ic = (gcode >> (2 * d)) & 3;
        if (sh[d] < 0 ? ic != 2 : ic != 0) return false;
    }
    return true;
}

template <int ND>
__device__ __forceinline__ bool any_shift(const int *sh) {
    bool a = false;
#pragma unroll
    for (int d = 0; d < ND; d++) a |= sh[d] != 0;
    return a;
}

/* The reference's FP64 predicate for a pair inside the FP32 band. */
template <int ND>
__device__ __noinline__ bool exact_pair(const DevCfg *__restrict__ cp, const DevState s, int a, int b, int sh0,
                                        int sh1, int sh2, double lim2, int strict) {
    const int sh[3] = {sh0, sh1, sh2};
    double dx[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < ND; d++)
        dx[d] = dsub(s.row(FD_R + d)[a], image_pos(s.row(FD_R + d)[b], sh[d], cp->rmin[d], cp->rmax[d]));
    const double r2 = exact_len2(dx, ND);
    if (lim2 > 0) return strict ? r2 < lim2 : r2 <= lim2;
    const double ha = s.row(FD_H)[a], hb = s.row(FD_H)[b];
    const double t = 2.0 * (ha > hb ? ha : hb);
    return r2 <= dmul(t, t);
}

/* ---------------------------------------------------------------------- */
/* P0 = (offset from own bucket origin, h), P1 = (vhat, mass; negated for
 * particles that are neither sph / sphBoundary nor DEM),
 * P2 = (dens, pdr2, porosity, 1/h), tg = type | gcode << 8 */
/* reference DEM bucket indices packed 10 bits per axis (biased by 512) */
constexpr int CP_BIAS = 512;

__device__ __forceinline__ int pack_cells(const int *k, int nd) {
    int p = 0;
    for (int d = 0; d < nd; d++) p |= ((k[d] + CP_BIAS) & 1023) << (10 * d);
    return p;
}

template <int ND>
__global__ void k_pack(DevCfg c, DevState s, const int *__restrict__ skey, const DevGlobals *__restrict__ g,
                       float4 *__restrict__ P0, float4 *__restrict__ P1, float4 *__restrict__ P2,
                       float4 *__restrict__ P0lo, int *__restrict__ tg, int4 *__restrict__ RC4, int with_rc,
                       float4 *__restrict__ DS, float4 *__restrict__ NB, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    tg[i] = (t & 0xff) | (s.irow(FI_GCODE)[i] << 8);
    if (t == T_DEAD) return;
    const int key = skey[i];
    float off[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
    int cc[3] = {0, 0, 0};
    const bool dem = c.liq_dem() && t == T_DEM;
    if (dem) {
        decode<ND>(key - g->n_sph_cells, c.ddims, cc);
    } else {
        const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
        decode<ND>(key, dims, cc);
    }
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const double o = s.row(FD_R + d)[i] - (dem ? dem_origin(c, d, cc[d]) : sph_origin(c, g, d, cc[d]));
        off[d] = (float)o;
        lo[d] = (float)(o - (double)off[d]);
    }
    {
        const double h = s.row(FD_H)[i];
        P0lo[i] = make_float4(lo[0], lo[1], lo[2], (float)(h - (double)(float)h));
    }
    float vh[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < ND; d++) vh[d] = (float)s.row(FD_VHAT + d)[i];
    P0[i] = make_float4(off[0], off[1], off[2], (float)s.row(FD_H)[i]);
    /* the mass of a particle that is neither sph / sphBoundary nor DEM is
     * stored negated: list readers take a neighbour's type from the sign and
     * load the type row only for those (walls) */
    const float mpk = (float)s.row(FD_MASS)[i];
    P1[i] = make_float4(vh[0], vh[1], vh[2], (is_sph_or_sphb(t) || dem) ? mpk : -mpk);
    /* a DEM particle's pdr2 slot holds its radius (the contact pre-test) */
    const double rad = s.row(FD_RADIUS)[i] > 0 ? s.row(FD_RADIUS)[i] : c.dem_radius;
    P2[i] = make_float4((float)s.row(FD_DENS)[i], (float)(t == T_DEM ? rad : s.row(FD_PDR2)[i]),
                        (float)s.row(FD_POR)[i], (float)s.row(FD_IH)[i]);
    if (is_boundary(t)) {
        float nv[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
        for (int k = 0; k < ND; k++) {
            nv[0][k] = (float)s.row(FD_N1 + k)[i];
            nv[1][k] = (float)s.row(FD_N2 + k)[i];
            nv[2][k] = ND == 3 ? (float)s.row(FD_N3 + k)[i] : 0.f;
        }
        NB[3 * i] = make_float4(nv[0][0], nv[0][1], nv[0][2], s.irow(FI_CONCAVE)[i] ? 1.f : -1.f);
        NB[3 * i + 1] = make_float4(nv[1][0], nv[1][1], nv[1][2], 0.f);
        NB[3 * i + 2] = make_float4(nv[2][0], nv[2][1], nv[2][2], 0.f);
    }
    if (dem) {
        /* the SPH bucket of a DEM particle and its FP32 offset there (calcFPI) */
        const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
        int k[3] = {0, 0, 0}, key = 0;
        float o[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < ND; d++) {
            const double r = s.row(FD_R + d)[i];
            int kd = c.periodic[d] ? (int)floor((r - c.dmin[d]) * g->rscell[d])
                                   : trunc_index(r, c.dmin[d], g->sr2, g->rsr2_f, 3.0);
            kd = kd < 0 ? 0 : (kd >= dims[d] ? dims[d] - 1 : kd);
            k[d] = kd;
            key = key * dims[d] + kd;
            o[d] = (float)(r - sph_origin(c, g, d, kd));
        }
        DS[i] = make_float4(o[0], o[1], o[2], __int_as_float(key));
    }
    if (with_rc) {
        /* reference DEM buckets (dem_getCellI) of the particle and, for DEM
         * particles, of its periodic images one period below / above */
        int k[3] = {0, 0, 0}, km[3] = {0, 0, 0}, kp[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < ND; d++) {
            const double r = s.row(FD_R + d)[i];
            k[d] = ref_dem_cell(r, c, d);
            if (dem && c.periodic[d]) {
                km[d] = ref_dem_cell(image_pos(r, -1, c.rmin[d], c.rmax[d]), c, d);
                kp[d] = ref_dem_cell(image_pos(r, 1, c.rmin[d], c.rmax[d]), c, d);
            }
        }
        RC4[i] = make_int4(pack_cells(k, ND), pack_cells(km, ND), pack_cells(kp, ND), 0);
    }
}

/* Coupling windows: for SPH bucket index i on axis d, the DEM buckets
 * [klo, khi] within Rc of it and the FP32 offset of its origin from the
 * origin of DEM bucket klo (one FP64 evaluation per bucket per rebuild). */
template <int ND>
__global__ void k_win(DevCfg c, const DevGlobals *__restrict__ g, int4 *__restrict__ win, int win_cap) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = t / win_cap, i = t - d * win_cap;
    if (d >= ND || i >= g->sdims[d]) return;
    const double lo = sph_origin(c, g, d, i);
    const double hi = lo + sph_width(c, g, d);
    int klo = (int)floor((lo - c.rc - c.dorig[d]) * c.rdcell[d]);
    int khi = (int)floor((hi + c.rc - c.dorig[d]) * c.rdcell[d]);
    if (!c.periodic[d]) {
        klo = max(klo, 0);
        khi = min(khi, c.ddims[d] - 1);
    }
    win[t] = make_int4(klo, khi, __float_as_int((float)(lo - (c.dorig[d] + klo * c.dcell[d]))), 0);
}

/* fields the DEM side gathers from fluid neighbours in calcFPI (sph.h:1708-1792):
 * Q0 = (fp+fb, fv.x), Q1 = (fv.y, fv.z, f.x, f.y), Q2 = (f.z, fdrag) */
__global__ void k_pack_fpi(DevState s, float4 *__restrict__ Q0, float4 *__restrict__ Q1, float4 *__restrict__ Q2,
                           int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[12];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        v[d] = (float)(s.row(FD_FP + d)[i] + s.row(FD_FB + d)[i]);
        v[3 + d] = (float)s.row(FD_FV + d)[i];
        v[6 + d] = (float)s.row(FD_F + d)[i];
        v[9 + d] = (float)s.row(FD_FDRAG + d)[i];
    }
    Q0[i] = make_float4(v[0], v[1], v[2], v[3]);
    Q1[i] = make_float4(v[4], v[5], v[6], v[7]);
    Q2[i] = make_float4(v[8], v[9], v[10], v[11]);
}

/* the reference's FP64 neighbour predicate, len2(ra - image(rb)) <= (2 max(ha, hb))^2
 * (dataLL.h neighbour traversal), evaluated without contraction */
template <int ND>
__device__ __forceinline__ bool exact_neighbour(const DevCfg &c, const DevState &s, int a, int b, const int *sh) {
    double dx[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < ND; d++)
        dx[d] = dsub(s.row(FD_R + d)[a], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
    const double r2 = exact_len2(dx, ND);
    const double ha = s.row(FD_H)[a], hb = s.row(FD_H)[b];
    const double t = 2.0 * (ha > hb ? ha : hb);
    return r2 <= dmul(t, t);
}

/* ---------------------------------------------------------------------- */
/* Half-width of the band around a cut-off T = R^2 inside which an FP32 r^2
 * built from bucket offsets cannot decide: each displacement component is
 * off by < 6 * 2^-24 L when L bounds the magnitudes of the offset terms, so
 * r^2 by < 1.25e-6 L max(L, R) + 1.8e-7 r^2, and T by < 1.8e-7 T. */
__device__ __forceinline__ float fp32_band(float T, float L2) { return fmaf(5e-7f, T, 1.5e-6f * fmaxf(L2, T)); }

constexpr int CENTER_CODE = 13 << B_BITS;

__device__ __forceinline__ void nl_decode_code(int code, int *o) {
    o[0] = code / 9 - 1;
    o[1] = (code / 3) % 3 - 1;
    o[2] = code % 3 - 1;
}

/* Double-float (hi + lo FP32) decision for one candidate near the cut-off:
 * +1 inside, -1 outside, 0 an FP64 tie.  Offsets, bucket size and h as hi+lo
 * pairs carry ~48 bits, so r^2 - (2h)^2 is known to ~1e-13 of (2h)^2 plus
 * ~1e-14 c^2 (c the bucket size); within 1e-12 of (2h)^2 + tol_abs only the
 * FP64 predicate decides. */
template <int ND>
__device__ __forceinline__ int nl_refine(const float4 pa, const float4 al, const float4 pb, const float4 bl,
                                         const int *o, const float *cell, const float *cell_lo, float tol_abs) {
    const float ah[3] = {pa.x, pa.y, pa.z}, bh[3] = {pb.x, pb.y, pb.z};
    const float alo[3] = {al.x, al.y, al.z}, blo[3] = {bl.x, bl.y, bl.z};
    float r2h = 0.f, r2l = 0.f;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        float s1v, e1, s2v, e2;
        two_sum(ah[d], -bh[d], s1v, e1);
        two_sum(s1v, -o[d] * cell[d], s2v, e2);
        const float lo = e1 + e2 + (alo[d] - blo[d]) - o[d] * cell_lo[d];
        float dh, dl;
        two_sum(s2v, lo, dh, dl);
        float p, pe;
        two_prod(dh, dh, p, pe);
        float t1, te;
        two_sum(r2h, p, t1, te);
        r2h = t1;
        r2l += te + pe + 2.f * dh * dl;
    }
    const bool amax = pa.w > pb.w || (pa.w == pb.w && al.w >= bl.w);
    const float hh = 2.f * (amax ? pa.w : pb.w), hl = 2.f * (amax ? al.w : bl.w);
    float Th, Te;
    two_prod(hh, hh, Th, Te);
    const float Tl = Te + 2.f * hh * hl;
    const float diff = (r2h - Th) + (r2l - Tl);
    if (fabsf(diff) <= 1e-12f * Th + tol_abs) return 0;
    return diff < 0.f ? 1 : -1;
}

/* ---------------------------------------------------------------------- */
/* Neighbour-list build.
 *
 * A warp takes 32 consecutive particles of the bucket order.  Buckets are
 * numbered with the last axis fastest, so those particles lie in one or two
 * runs of consecutive buckets along that axis (a "column").  For each run
 * the warp stages the candidates of the union of the runs' 3^d stencils --
 * 3^(d-1) neighbour columns x the run's z-range +-1 -- in shared memory,
 * with positions moved into the run's frame (coalesced loads; the periodic
 * image filter is applied once per candidate), then every lane tests all
 * staged candidates with broadcast shared-memory reads.  Sharing the stencil
 * across a run keeps all 32 lanes busy whatever the bucket occupancy.
 *
 * FP32 error bound of the test (L = largest offset magnitude in the frame,
 * R = 2 max(ha, hb)): each displacement component carries < 6 * 2^-24 L, so
 * r^2 is off by < 1.25e-6 L max(L, R) + 1.8e-7 r^2 and the cut-off
 * 4 max(ha^2, hb^2) by < 1.8e-7 of itself.  Candidates closer than
 * fp32_band(T, L^2) to the cut-off are recorded per particle (up to NL_QB)
 * and decided by k_band_fix; beyond that they are decided inline in FP64. */
constexpr int NL_WARPS = 8;
constexpr int NL_CAP = 256;   /* staged candidates per warp before a flush */
constexpr int NL_QB = 32;     /* band candidates recorded per particle */

__device__ __forceinline__ int code_stride(int d) { return d == 0 ? 9 : (d == 1 ? 3 : 1); }

/* FP64 decision of list entry e of particle a (bucket cc), out of line */
template <int ND>
__device__ __noinline__ bool exact_from_code(const DevCfg &c, const DevState &s, const DevGlobals *g, int a, int e,
                                             const int *cc) {
    int o[3], sh[3] = {0, 0, 0};
    nl_decode_code(e >> B_BITS, o);
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const int t = cc[d] + o[d];
        sh[d] = t < 0 ? -1 : (t >= dims[d] ? 1 : 0);
    }
    return exact_neighbour<ND>(c, s, a, e & B_MASK, sh);
}

/* FP64 decision of list entry e of particle a, its bucket from the key row */
template <int ND>
__device__ __noinline__ bool exact_from_key(const DevCfg &c, const DevState &s, const DevGlobals *g,
                                            const int *skey, int a, int e) {
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    int cc[3] = {0, 0, 0};
    decode<ND>(skey[a], dims, cc);
    return exact_from_code<ND>(c, s, g, a, e, cc);
}

/* Neighbour lists: slot j of particle a, in tiles of 32 particles x 8
 * entries -- each particle's 8 entries contiguous, the 32 particles' groups
 * back to back -- so a warp of consecutive particles reads 8 entries each
 * with two coalesced int4 loads and the build writes a particle's entries in
 * runs.  maxn (the list depth) is a multiple of 8. */
__device__ __forceinline__ int64_t nl_at(int64_t a, int j, int64_t maxn) {
    return ((a >> 5) * maxn + (j & ~7)) * 32 + ((a & 31) << 3) + (j & 7);
}

/* lane bits [lo, hi), 0 <= lo <= hi <= 32 */
__device__ __forceinline__ unsigned lane_range(int lo, int hi) {
    const unsigned up = hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u);
    const unsigned dn = lo >= 32 ? 0xffffffffu : ((1u << lo) - 1u);
    return up & ~dn;
}

template <int ND, bool COUNT>
__global__ void __launch_bounds__(NL_WARPS * 32, 3) k_nlist(DevCfg c, DevState s, const int *__restrict__ start,
                                                         const int *__restrict__ skey, DevGlobals *__restrict__ g,
                                                         const float4 *__restrict__ P0, const int *__restrict__ tg,
                                                         int *__restrict__ nbr, int *__restrict__ ncnt, int maxn,
                                                         int64_t ld, int2 *__restrict__ bandq,
                                                         int *__restrict__ bandn) {
    constexpr int Z = ND - 1;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ float4 s_pos[NL_WARPS][NL_CAP + 32];
    __shared__ int s_ent[NL_WARPS][NL_CAP + 32];
    __shared__ unsigned char s_zr[NL_WARPS][NL_CAP];
    __shared__ float4 s_own[NL_WARPS][32];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float4 *cpos = s_pos[w];
    int *cent = s_ent[w];
    unsigned char *czr = s_zr[w];
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nsc = g->n_sph_cells;
    const int n_t = start[nsc];
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    const int zdim = dims[Z];
    float cell[3];
    float l_other = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        cell[d] = (float)(c.periodic[d] ? g->scell[d] : g->sr2);
        if (d < Z) l_other = fmaxf(l_other, 2.f * cell[d]);
    }
    const float cz = cell[Z];
    int code_fixed = 0;
#pragma unroll
    for (int d = ND; d < 3; d++) code_fixed += code_stride(d);
    const int zstride = code_stride(Z) << B_BITS;
    const int self_e = CENTER_CODE;
    const float supp = (float)(2.0 * g->sr) * (1.f + 1e-5f) + 1e-5f * cz;
    const float K_HI = 4.f * (1.f + 5e-7f), K_LO = 4.f * (1.f - 5e-7f);

    for (int t0 = (blockIdx.x * NL_WARPS + w) * 32; t0 < n_t; t0 += NL_WARPS * gridDim.x * 32) {
        const int a = t0 + lane;
        /* the warp's 32 particles share one column of list tiles: entry j of
         * particle t0 + i sits at tiles + (j & ~7) * 32 + i * 8 + (j & 7) */
        int *const tiles = nbr + (int64_t)(t0 >> 5) * maxn * 32;
        bool act = false;
        int key = 0;
        if (a < n_t) {
            key = skey[a];
            act = is_sph_or_sphb(tg[a] & 0xff);
        }
        int cc[3] = {0, 0, 0};
        decode<ND>(key, dims, cc);
        const int col = key / zdim;
        float4 pa0 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (act) pa0 = P0[a];
        int cnt = 0, nb = 0;
        unsigned pending = __ballot_sync(FULL, act);
        while (pending) {
            /* a run: lanes in the leader's column within 3 buckets of it */
            const int leader = __ffs(pending) - 1;
            const int lcol = __shfl_sync(FULL, col, leader);
            const int zmin = __shfl_sync(FULL, cc[Z], leader);
            const unsigned gmask = __ballot_sync(FULL, act && col == lcol && cc[Z] <= zmin + 2) & pending;
            pending &= ~gmask;
            const int zmax = __shfl_sync(FULL, cc[Z], 31 - __clz(gmask));
            int ccol[3] = {0, 0, 0};
#pragma unroll
            for (int d = 0; d < Z; d++) ccol[d] = __shfl_sync(FULL, cc[d], leader);
            const bool mine = (gmask >> lane) & 1u;
            /* this lane's particle in the run's frame; others sit far away */
            float pv[3] = {1e30f, 1e30f, 1e30f};
            float ha2 = 0.f;
            if (mine) {
                pv[0] = pa0.x;
                pv[1] = pa0.y;
                pv[2] = pa0.z;
                pv[Z] += (float)(cc[Z] - zmin) * cz;
                ha2 = pa0.w * pa0.w;
            }
            const int lane_zr = cc[Z] - zmin + 1;
            const float L = fmaxf(l_other, (float)(zmax - zmin + 2) * cz);
            const float EPS = 1.5e-6f * L * L;
            /* the run's extent on the last axis, widened by the largest support
             * 2 sr >= 2 max(h) and a rounding margin: nothing outside is a neighbour */
            float zt_lo = mine ? pv[Z] : 1e30f, zt_hi = mine ? pv[Z] : -1e30f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                zt_lo = fminf(zt_lo, __shfl_xor_sync(FULL, zt_lo, o));
                zt_hi = fmaxf(zt_hi, __shfl_xor_sync(FULL, zt_hi, o));
            }
            zt_lo -= supp;
            zt_hi += supp;
            int nst = 0;

            /* Test the staged candidates 32 at a time, branch-free: one bit per
             * candidate that passes the widened FP32 test (the staged set is
             * padded to a multiple of 32 with far-away entries; each staged w
             * holds the candidate's own threshold K_HI h_b^2 + EPS).  The warp
             * then writes the passing entries of all its lanes together: the
             * t-th entry of the chunk goes to the lane whose prefix of pass
             * counts covers t, and each particle's entries land in consecutive
             * slots of its 8-entry list tiles, so the stores coalesce.  The
             * particle itself and band candidates outside the particle's own
             * stencil leave a hole (-1), which every reader skips. */
            const float thr_a = fmaf(ha2, K_HI, EPS);
            s_own[w][lane] = make_float4(pv[0], pv[1], pv[2], ha2);
            __syncwarp();
            const int my_zr = lane_zr;
            auto evaluate = [&]() {
                if (lane < ((32 - (nst & 31)) & 31)) {
                    cpos[nst + lane] = make_float4(-1e30f, -1e30f, -1e30f, 0.f);
                    cent[nst + lane] = 0;
                }
                __syncwarp();
                for (int j0 = 0; j0 < nst; j0 += 32) {
                    unsigned pm = 0u;
#pragma unroll 8
                    for (int jj = 0; jj < 32; jj++) {
                        const float4 q = cpos[j0 + jj];
                        const float dx = pv[0] - q.x;
                        const float dy = ND > 1 ? pv[1] - q.y : 0.f;
                        const float dz = ND > 2 ? pv[2] - q.z : 0.f;
                        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                        pm |= (r2 <= fmaxf(thr_a, q.w) ? 1u : 0u) << jj;
                    }
                    const int c_i = __popc(pm);
                    if (COUNT) {
                        cnt += c_i;
                        continue;
                    }
                    int incl = c_i;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o) incl += v;
                    }
                    const int T = __shfl_sync(FULL, incl, 31);
                    const int my_ex = incl - c_i;
                    for (int base = 0; base < T; base += 32) {
                        const int t = base + lane;
                        /* owner: the first lane whose inclusive count exceeds t */
                        int i = 0;
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1) {
                            const int v = __shfl_sync(FULL, incl, i + step - 1);
                            if (v <= t) i += step;
                        }
                        const unsigned pmi = __shfl_sync(FULL, pm, i);
                        const int exi = __shfl_sync(FULL, my_ex, i);
                        const int cni = __shfl_sync(FULL, cnt | (nb << 16), i);
                        const int zri = __shfl_sync(FULL, my_zr, i);
                        const float4 own = s_own[w][i];
                        const float pxi = own.x, pyi = own.y, pzi = own.z, h2i = own.w;
                        const bool on = t < T;
                        int e = -1, slot = 0, j = 0;
                        const int ai = t0 + i;
                        bool band = false;
                        if (on) {
                            /* the r-th set bit of the owner's mask */
                            const int r = t - exi;
                            unsigned m = pmi;
                            int bit = 0, rr = r;
#pragma unroll
                            for (int w2 = 16; w2 > 0; w2 >>= 1) {
                                const int cl = __popc(m & ((1u << w2) - 1u));
                                if (rr >= cl) {
                                    rr -= cl;
                                    m >>= w2;
                                    bit += w2;
                                }
                            }
                            j = j0 + bit;
                            slot = (cni & 0xffff) + r;
                            e = (int)((unsigned)cent[j] + (unsigned)(1 - zri) * (unsigned)zstride);
                            if (e == (ai | self_e)) {
                                e = -1; /* the particle itself */
                            } else {
                                const float4 q = cpos[j];
                                const float dx = pxi - q.x;
                                const float dy = ND > 1 ? pyi - q.y : 0.f;
                                const float dz = ND > 2 ? pzi - q.z : 0.f;
                                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                                band = r2 >= fmaf(fmaxf(h2i, q.w * (1.f / K_HI)), K_LO, -2.f * EPS);
                            }
                        }
                        const unsigned bb = __ballot_sync(FULL, band);
                        if (band) {
                            /* buckets are at least 2h wide, so a candidate outside this
                             * particle's own 3^d stencil is at least 2h away: it can only
                             * pass the FP32 test inside the band, and is no neighbour */
                            const bool in_stencil = (unsigned)((int)czr[j] - zri + 1) <= 2u;
                            const int qb = (cni >> 16) + __popc(bb & lane_range(max(exi - base, 0), lane));
                            if (qb < NL_QB) {
                                bandq[(int64_t)ai * NL_QB + qb] =
                                    in_stencil && slot < maxn ? make_int2(e, slot) : make_int2(-1, -1);
                                e = in_stencil ? (e | (int)0x80000000u) : -1;
                            } else if (!in_stencil || !exact_from_key<ND>(c, s, g, skey, ai, e)) {
                                e = -1; /* record full: decided here (slow but exact) */
                            }
                        }
                        if (on && slot < maxn) tiles[((slot & ~7) << 5) + (i << 3) + (slot & 7)] = e;
                        /* band records of this lane's own entries in this round
                         * (bb is warp-uniform and almost always empty) */
                        if (bb)
                            nb += __popc(bb & lane_range(min(max(my_ex - base, 0), 32),
                                                         min(max(my_ex + c_i - base, 0), 32)));
                    }
                    cnt += c_i;
                }
                __syncwarp();
                nst = 0;
            };

            /* Range table, one lane per (neighbour column, period piece): the
             * column's buckets zmin-1 .. zmax+1 cut at the periodic seam into at
             * most 3 runs of consecutive keys.  All lanes load their bucket range
             * at once; the candidates of all ranges are then gathered flat. */
            constexpr int NCOL = Z == 2 ? 9 : (Z == 1 ? 3 : 1);
            int r_b0 = 0, r_cnt = 0, r_lin = 0, r_zoff = 0, r_code = 0, r_sh = 0;
            float r_ox = 0.f, r_oy = 0.f;
            if (lane < 3 * NCOL) {
                const int colidx = lane / 3, wz = lane % 3 - 1;
                int o[2] = {0, 0};
                if (Z == 2) {
                    o[0] = colidx / 3 - 1;
                    o[1] = colidx % 3 - 1;
                } else if (Z == 1) {
                    o[0] = colidx - 1;
                }
                bool ok = wz == 0 || c.periodic[Z];
                int col_lin = 0, code_o = code_fixed, shp = 0;
#pragma unroll
                for (int d = ND; d < 3; d++) shp |= 1 << (2 * d); /* unused axes: no shift */
                float off[2] = {0.f, 0.f};
#pragma unroll
                for (int d = 0; d < Z; d++) {
                    int t = ccol[d] + o[d], shd = 0;
                    if (t < 0) {
                        ok = ok && c.periodic[d];
                        t += dims[d];
                        shd = -1;
                    } else if (t >= dims[d]) {
                        ok = ok && c.periodic[d];
                        t -= dims[d];
                        shd = 1;
                    }
                    col_lin = col_lin * dims[d] + t;
                    code_o += (o[d] + 1) * code_stride(d);
                    off[d] = (float)o[d] * cell[d];
                    shp |= (shd + 1) << (2 * d);
                }
                shp |= (wz + 1) << (2 * Z);
                /* unwrapped z range of this piece */
                const int zlo = max(zmin - 1, wz * zdim), zhi = min(zmax + 1, (wz + 1) * zdim - 1);
                if (ok && zlo <= zhi) {
                    r_lin = col_lin * zdim + (zlo - wz * zdim);
                    r_b0 = start[r_lin];
                    r_cnt = start[r_lin + (zhi - zlo) + 1] - r_b0;
                    r_zoff = zlo - zmin;
                    r_code = code_o << B_BITS;
                    r_sh = shp;
                    r_ox = off[0];
                    r_oy = off[1];
                    /* buckets hold their particles sorted on the last axis, so the
                     * run is sorted there: keep only [zt_lo, zt_hi] (binary search) */
                    int lo = 0, hi = r_cnt;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1, k = r_b0 + mid;
                        const float4 q = P0[k];
                        const float z = (Z == 0 ? q.x : (Z == 1 ? q.y : q.z)) + (float)(r_zoff + skey[k] - r_lin) * cz;
                        if (z < zt_lo) lo = mid + 1;
                        else hi = mid;
                    }
                    const int first = lo;
                    hi = r_cnt;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1, k = r_b0 + mid;
                        const float4 q = P0[k];
                        const float z = (Z == 0 ? q.x : (Z == 1 ? q.y : q.z)) + (float)(r_zoff + skey[k] - r_lin) * cz;
                        if (z <= zt_hi) lo = mid + 1;
                        else hi = mid;
                    }
                    r_b0 += first;
                    r_cnt = lo - first;
                }
            }
            /* exclusive prefix of the range sizes over the lanes */
            int r_excl = r_cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, r_excl, o);
                if (lane >= o) r_excl += v;
            }
            const int total = __shfl_sync(FULL, r_excl, 31);
            r_excl -= r_cnt;

            for (int t = 0;;) {
              for (; t < total && nst + 32 <= NL_CAP; t += 32) {
                const int j = t + lane;
                /* the range holding flat index j: the last lane with excl <= j */
                int src = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int e = __shfl_sync(FULL, r_excl, src + step);
                    if (e <= j) src += step;
                }
                const int b0 = __shfl_sync(FULL, r_b0, src), ex = __shfl_sync(FULL, r_excl, src);
                const int lin = __shfl_sync(FULL, r_lin, src), zoff = __shfl_sync(FULL, r_zoff, src);
                const int code = __shfl_sync(FULL, r_code, src), shp = __shfl_sync(FULL, r_sh, src);
                const float ox = __shfl_sync(FULL, r_ox, src), oy = __shfl_sync(FULL, r_oy, src);
                bool valid = j < total;
                float4 pb = make_float4(0.f, 0.f, 0.f, 0.f);
                int k = 0, zrel = 0;
                if (valid) {
                    k = b0 + (j - ex);
                    pb = P0[k];
                    zrel = zoff + (skey[k] - lin);
                    if (shp != 0x15) {
                        const int shv[3] = {(shp & 3) - 1, ((shp >> 2) & 3) - 1, ((shp >> 4) & 3) - 1};
                        valid = img_ok<ND>(tg[k] >> 8, shv);
                    }
                }
                const unsigned m = __ballot_sync(FULL, valid);
                if (valid) {
                    const int pos = nst + __popc(m & lt_mask);
                    float qv[3] = {pb.x, pb.y, pb.z};
                    if (Z > 0) qv[0] += ox;
                    if (Z > 1) qv[1] += oy;
                    qv[Z] += (float)zrel * cz;
                    cpos[pos] = make_float4(qv[0], qv[1], qv[2], fmaf(pb.w * pb.w, K_HI, EPS));
                    /* k | code of the candidate's bucket relative to the run's
                     * first bucket - 1; evaluate adds the lane's own offset */
                    cent[pos] = (int)((unsigned)(k | code) + (unsigned)(zrel + 1) * (unsigned)zstride);
                    czr[pos] = (unsigned char)(zrel + 1);
                }
                nst += __popc(m);
              }
              evaluate();
              if (t >= total) break;
            }
        }
        if (act) {
            ncnt[a] = COUNT ? cnt : min(cnt, maxn);
            if (!COUNT) {
                bandn[a] = min(nb, NL_QB);
                /* stored counts never exceed the list depth; an overflow is an error */
                if (cnt > maxn) set_err(g, SPHDEM_ERR_CAPACITY, cnt);
            }
        } else if (!COUNT && a < n_t) {
            bandn[a] = 0;
        }
    }
}

/* Decide the recorded band candidates of every particle: the double-float
 * refinement settles all but FP64 ties, which take the reference's FP64
 * predicate.  Keep (clear the pending bit) or mark the list slot invalid (-1). */
template <int ND>
__global__ void k_band_fix(DevCfg c, DevState s, const DevGlobals *__restrict__ g, const int *__restrict__ start,
                           const int *__restrict__ skey, const float4 *__restrict__ P0,
                           const float4 *__restrict__ P0lo, const int2 *__restrict__ bandq,
                           const int *__restrict__ bandn, int *__restrict__ nbr, int64_t ld) {
    const int n_t = start[g->n_sph_cells];
    float cell[3], cell_lo[3];
    float cmax = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double cw = c.periodic[d] ? g->scell[d] : g->sr2;
        cell[d] = (float)cw;
        cell_lo[d] = (float)(cw - (double)cell[d]);
        if (d < ND) cmax = fmaxf(cmax, cell[d]);
    }
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n_t; a += gridDim.x * blockDim.x) {
        const int nb = bandn[a];
        if (nb == 0) continue;
        int cc[3] = {0, 0, 0};
        decode<ND>(skey[a], dims, cc);
        const float4 pa = P0[a], al = P0lo[a];
        for (int k = 0; k < nb; k++) {
            const int2 it = bandq[(int64_t)a * NL_QB + k];
            if (it.y < 0) continue; /* a blank record */
            const int e = it.x, b = e & B_MASK;
            int o[3];
            nl_decode_code(e >> B_BITS, o);
            int dec = nl_refine<ND>(pa, al, P0[b], P0lo[b], o, cell, cell_lo, 1e-13f * cmax * cmax);
            /* an FP64 tie: the reference's predicate on the periodic image */
            if (dec == 0) dec = exact_from_code<ND>(c, s, g, a, e, cc) ? 1 : -1;
            nbr[nl_at(a, it.y, ld)] = dec > 0 ? e : -1;
        }
    }
}

__device__ __forceinline__ void load_cell32(const DevCfg &c, const DevGlobals *g, float *cell) {
#pragma unroll
    for (int d = 0; d < 3; d++) cell[d] = (float)(c.periodic[d] ? g->scell[d] : g->sr2);
}

/* The 27 stencil shifts o * bucket size, indexed by the list entry's code,
 * in shared memory: one load per pair instead of a decode and three
 * int-to-float conversions.  Every thread of the block must call this. */
__device__ __forceinline__ const float4 *stencil_shifts(const DevCfg &c, const DevGlobals *g) {
    __shared__ float4 tab[27];
    if (threadIdx.x < 27) {
        const int code = threadIdx.x;
        const float o0 = (float)(code / 9 - 1), o1 = (float)((code / 3) % 3 - 1), o2 = (float)(code % 3 - 1);
        float cell[3];
        load_cell32(c, g, cell);
        tab[code] = make_float4(o0 * cell[0], o1 * cell[1], o2 * cell[2], 0.f);
    }
    __syncthreads();
    return tab;
}

template <int ND>
__device__ __forceinline__ void nb_delta_t(int e, const float4 *tab, float4 pa, float4 pb, float *d) {
    const float4 sft = tab[e >> B_BITS];
    d[0] = pa.x - pb.x - sft.x;
    d[1] = ND > 1 ? pa.y - pb.y - sft.y : 0.f;
    d[2] = ND > 2 ? pa.z - pb.z - sft.z : 0.f;
}

/* ---------------------------------------------------------------------- */
template <int ND>
__global__ void __launch_bounds__(BLK) k_omega_eos(DevCfg c, DevState s, const DevGlobals *__restrict__ g,
                                                   const float4 *__restrict__ P0, const float4 *__restrict__ P1,
                                                   float4 *__restrict__ P2, const int *__restrict__ tg,
                                                   const int *__restrict__ nbr, const int *__restrict__ ncnt,
                                                   int64_t ld, int64_t n, int do_omega, int do_eos,
                                                   float *__restrict__ om32) {
    const float4 *shift = stencil_shifts(c, g);
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    if (do_omega) {
        const float wcon = (float)c.wcon;
        const float4 pa = P0[a];
        const float iha = 1.f / pa.w;
        const float ihna = powi<ND>(iha);
        const float pd_coef = ND * ihna * iha;
        Kahan om;
        om.init(-P1[a].w * pd_coef * wK32(0.f, wcon));
        const int cnt = ncnt[a];
        /* 8 entries at a time from the particle's list tiles (two int4 loads) */
        const int4 *tile = reinterpret_cast<const int4 *>(nbr + nl_at(a, 0, ld));
        int4 q0 = make_int4(-1, -1, -1, -1), q1 = q0;
#pragma unroll 2
        for (int j = 0; j < cnt; j++) {
            if ((j & 7) == 0) {
                q0 = __ldg(tile + (j >> 3) * 64);
                q1 = __ldg(tile + (j >> 3) * 64 + 1);
            }
            const int e = q0.x;
            q0 = make_int4(q0.y, q0.z, q0.w, q1.x);
            q1 = make_int4(q1.y, q1.z, q1.w, -1);
            if (e < 0) continue;
            const int b = e & B_MASK;
            const float4 pb = P0[b];
            const float mb = fabsf(P1[b].w);
            const int tb = tg[b] & 0xff;
            float d[3];
            nb_delta_t<ND>(e, shift, pa, pb, d);
            const float q = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * iha;
            const float pdkh = -q * wdK32(q, wcon) * iha;
            if (is_sph_or_sphb(tb)) om.add(mb * (ihna * pdkh - pd_coef * wK32(q, wcon)));
        }
        /* Omega = 1 + h*sum/(rho*NDIM): an O(1) number, FP32 is ample */
        const float omega = 1.f + pa.w * om.s / (P2[a].x * ND);
        s.row(FD_OMEGA)[a] = omega;
        om32[a] = omega;
    }
    if (do_eos) {
        /* FP64: p = PRB((rho/rho0)^7 - 1) cancels; one FP64 reciprocal by
         * an FP32 estimate and a Newton step, integer powers */
        const double densa = s.row(FD_DENS)[a];
        const double rho0 = c.liq_dem() ? c.refd * s.row(FD_POR)[a] : c.refd;
        double r0 = (double)(1.0f / (float)rho0);
        r0 = r0 * (2.0 - rho0 * r0);
        const double x = densa * r0;
        double xg;
        if (!c.liq_dem() || c.gamma == 7.0) {
            const double x2 = x * x;
            xg = x2 * x2 * x2 * x;
        } else {
            xg = pow(x, c.gamma);
        }
        double rd = (double)(1.0f / (float)densa);
        rd = rd * (2.0 - densa * rd);
        const double press = c.prb * (xg - 1.0);
        const double pdr2 = press * (rd * rd);
        s.row(FD_PRESS)[a] = press;
        s.row(FD_PDR2)[a] = pdr2;
        float4 p2 = P2[a];
        p2.y = (float)pdr2;
        p2.z = (float)s.row(FD_POR)[a];
        P2[a] = p2;
    }
}

/* ---------------------------------------------------------------------- */
__device__ __forceinline__ void block_min_atomic(float v, unsigned long long *target) {
    __shared__ float smin[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) smin[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? smin[lane] : FLT_MAX;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v < FLT_MAX) atomic_min_pos(target, (double)v);
    }
}

/* boundary force of sph.h:736-918 in FP32 (b is a repulsive boundary particle) */
template <int ND>
__device__ __noinline__ void boundary32(const DevCfg *__restrict__ cp, const float4 *__restrict__ NB, int b, float d0,
                                        float d1, float d2, float r, float dv0, float dv1, float dv2, float ma, float mb,
                                        float *fbx) {
    const DevCfg &c = *cp;
    const float d[3] = {d0, d1, d2}, dv[3] = {dv0, dv1, dv2};
    const float4 N1 = NB[3 * b], N2 = NB[3 * b + 1], N3 = NB[3 * b + 2];
    const float n1[3] = {N1.x, N1.y, N1.z}, n2[3] = {N2.x, N2.y, N2.z}, nt[3] = {N3.x, N3.y, N3.z};
    float np[3];
    if (n2[0] == 0.f && n2[1] == 0.f && n2[2] == 0.f) {
        for (int k = 0; k < 3; k++) np[k] = n1[k];
    } else {
        const float rd1 = d[0] * n1[0] + d[1] * n1[1] + d[2] * n1[2];
        const float rd2 = d[0] * n2[0] + d[1] * n2[1] + d[2] * n2[2];
        const float rnt = r * r * (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) - rd1 * rd2;
        if (rnt <= 0.f) {
            for (int k = 0; k < 3; k++) np[k] = d[k] / r;
        } else {
            const float con = N1.w;
            for (int k = 0; k < 3; k++) np[k] = con * (rd1 - rd2) > 0.f ? n1[k] : n2[k];
        }
    }
    const float rperp = np[0] * d[0] + np[1] * d[1] + np[2] * d[2];
    const float rt0 = d[0] - rperp * np[0], rt1 = d[1] - rperp * np[1], rt2 = d[2] - rperp * np[2];
    const float rdelp = c.f_rdelp;
    float pt0, pt1;
    if (ND == 3) {
        pt0 = fabsf(rt0 * nt[0] + rt1 * nt[1] + rt2 * nt[2]);
        const float cx = rt1 * nt[2] - rt2 * nt[1], cy = rt2 * nt[0] - rt0 * nt[2], cz = rt0 * nt[1] - rt1 * nt[0];
        pt1 = sqrtf(cx * cx + cy * cy + cz * cz);
    } else {
        pt0 = sqrtf(rt0 * rt0 + rt1 * rt1);
        pt1 = 0.f;
    }
    const float pd0 = pt0 * rdelp, pd1 = pt1 * rdelp;
    if (!(pd0 <= 1.f && pd1 <= 1.f)) return;
    const float pif = c.f_pi, c0 = c.f_c0;
    const float pesky = 0.25f * (1.f + cosf(pif * pd0)) * (1.f + cosf(pif * pd1));
    const float q = fabsf(rperp) * c.f_rpsep;
    if (!(q < 2.f)) return;
    const int beta = (d[0] * dv[0] + d[1] * dv[1] + d[2] * dv[2]) < 0.f ? 1 : 0;
    const float bigA = 0.01f * c0 * c0 - beta * c0 * (dv[0] * np[0] + dv[1] * np[1] + dv[2] * np[2]);
    const float bfact = 1.f / fabsf(rperp);
    const float QIN = 2.f / 3.f;
    float bforce;
    if (q <= QIN) bforce = bfact * QIN;
    else if (q <= 1.f) bforce = bfact * (2.f * q - 1.5f * q * q);
    else bforce = bfact * 0.5f * (2.f - q) * (2.f - q);
    const float sc = (rperp < 0.f ? -1.f : 1.f) * (2.f * ma / (ma + mb)) * bigA * bforce * pesky;
    for (int k = 0; k < 3; k++) fbx[k] = sc * np[k];
}

/* ---------------------------------------------------------------------- */
/* Neighbour-record staging for the list consumers (TMA bulk copies).
 *
 * A block takes consecutive particles of the bucket order, so most of them
 * lie in one column of buckets along the last axis, and their neighbours in
 * the 3^(d-1) columns around it, over the block's bucket range on the last
 * axis +- one bucket.  Each of those column ranges is a contiguous run of
 * particle slots, so its packed records (P0, P1, P2) are copied global ->
 * shared with one cp.async.bulk per array, completing on one mbarrier.  A
 * list entry's stencil code names its neighbour column, so its record is
 * found in shared memory when its slot lies in that column's staged range,
 * else (another column of the block, a periodic image on the last axis, a
 * range cut at the capacity) read from global memory. */
constexpr int ST_CAP = 1536;    /* staged records per block (2 or 3 x 16 B each) */
constexpr int ST_MAXSLOT = 9;   /* neighbour columns: 3^(d-1) */

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

/* bounded wait for phase 0 of the staging barrier: false after the limit */
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar) {
    for (int it = 0; it < (1 << 22); it++)
        if (mbar_try_wait(bar, 0)) return true;
    return false;
}

struct Staged {
    const float4 *S0, *S1, *S2;
    const int *lo, *num, *base;
    bool ok;
};

/* the neighbour column of a stencil code (3D: code / 3, 2D: code / 9) */
template <int ND>
__device__ __forceinline__ int st_slot(int code) {
    return ND == 3 ? code / 3 : (ND == 2 ? code / 9 : 0);
}

/* Called by every thread of the block.  a0: the block's first slot, n_t:
 * the particles in SPH buckets (sorted by bucket key). */
template <int ND, int NARR>
__device__ Staged stage_neighbours(const DevCfg &c, DevGlobals *g, const int *__restrict__ start,
                                   const int *__restrict__ skey, const float4 *__restrict__ P0,
                                   const float4 *__restrict__ P1, const float4 *__restrict__ P2, int64_t a0,
                                   int n_t, float4 *smem) {
    constexpr int Z = ND - 1;
    constexpr int NS = ND == 3 ? 9 : (ND == 2 ? 3 : 1);
    __shared__ int s_lo[ST_MAXSLOT], s_num[ST_MAXSLOT], s_base[ST_MAXSLOT];
    __shared__ int s_col, s_zmin, s_zmax;
    __shared__ __align__(8) unsigned long long s_bar;
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    const int zdim = dims[Z];
    if (threadIdx.x == 0) {
        s_col = skey[a0] / zdim;
        s_zmin = INT_MAX;
        s_zmax = -1;
        mbar_init(&s_bar, 1);
    }
    __syncthreads();
    const int64_t a = a0 + threadIdx.x;
    if (a < n_t) {
        const int key = skey[a];
        if (key / zdim == s_col) {
            atomicMin(&s_zmin, key % zdim);
            atomicMax(&s_zmax, key % zdim);
        }
    }
    __syncthreads();
    if (threadIdx.x < NS) {
        const int t = threadIdx.x;
        int o[2] = {0, 0}, cc[2] = {0, 0};
        if (ND == 3) {
            o[0] = t / 3 - 1;
            o[1] = t % 3 - 1;
            cc[0] = s_col / dims[1];
            cc[1] = s_col % dims[1];
        } else if (ND == 2) {
            o[0] = t - 1;
            cc[0] = s_col;
        }
        bool ok = true;
        int col = 0;
#pragma unroll
        for (int d = 0; d < Z; d++) {
            int x = cc[d] + o[d];
            if (x < 0 || x >= dims[d]) {
                ok = ok && c.periodic[d];
                x = x < 0 ? x + dims[d] : x - dims[d];
            }
            col = col * dims[d] + x;
        }
        const int zlo = max(s_zmin - 1, 0), zhi = min(s_zmax + 1, zdim - 1);
        int lo = 0, num = 0;
        if (ok && zlo <= zhi) {
            lo = start[col * zdim + zlo];
            num = start[col * zdim + zhi + 1] - lo;
        }
        s_lo[t] = lo;
        s_num[t] = num;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int base = 0;
        for (int t = 0; t < NS; t++) {
            const int num = min(s_num[t], ST_CAP - base);
            s_num[t] = num;
            s_base[t] = base;
            base += num;
        }
        mbar_expect_tx(&s_bar, (unsigned)(NARR * 16 * base));
        for (int t = 0; t < NS; t++) {
            const int num = s_num[t];
            if (num <= 0) continue;
            const unsigned bytes = (unsigned)(16 * num);
            bulk_g2s(smem + s_base[t], P0 + s_lo[t], bytes, &s_bar);
            bulk_g2s(smem + ST_CAP + s_base[t], P1 + s_lo[t], bytes, &s_bar);
            if (NARR > 2) bulk_g2s(smem + 2 * ST_CAP + s_base[t], P2 + s_lo[t], bytes, &s_bar);
        }
    }
    __syncthreads();
    Staged st;
    st.S0 = smem;
    st.S1 = smem + ST_CAP;
    st.S2 = smem + 2 * ST_CAP;
    st.lo = s_lo;
    st.num = s_num;
    st.base = s_base;
    bool ok = mbar_wait_bounded(&s_bar);
    if (!ok) {
        /* gave up: record it, and keep the block alive (again bounded) until
         * the copies into its shared memory have landed */
        set_err(g, SPHDEM_ERR_TIMEOUT, 1);
        mbar_wait_bounded(&s_bar);
    }
    /* the whole block gives up together */
    st.ok = !__syncthreads_or(!ok);
    return st;
}

/* Physics classes the force pass is specialised on (so that the unused
 * viscosity forms, accumulators and branches compile away): the coupled
 * sedimentation form (Morris viscosity, VAR_H_CORRECTION, no anticlumping),
 * the dam-break form (artificial viscosity, constant h, no anticlumping),
 * and every other combination read from the configuration. */
enum : int { PHYS_GENERIC = 0, PHYS_MORRIS_VARH = 1, PHYS_ARTIFICIAL = 2, PHYS_CG = 3 };

/* CORRECTED_GRADIENT in FP32 (sph.h:325-326): the corrected gradient of a
 * pair is invM_a ((dr F - sumGrad_a/sum_a) / sum_a); invM_a, sumGrad_a and
 * sum_a come from calcInvM (FP64, k_invm) once per rebuild and enter each
 * owner's pair loop as M = invM_a / sum_a and cs = sumGrad_a / sum_a. */
template <int ND>
struct Cg32 {
    float m[ND * ND], cs[ND];
    __device__ __forceinline__ void load(const double *cg, int64_t cap, int64_t a) {
        const double sum = cg[CG_S * cap + a];
#pragma unroll
        for (int k = 0; k < ND * ND; k++) m[k] = (float)(cg[(CG_M + k) * cap + a] / sum);
#pragma unroll
        for (int d = 0; d < ND; d++) cs[d] = (float)cg[(CG_C + d) * cap + a];
    }
    /* out = M (d F - cs) */
    __device__ __forceinline__ void apply(const float *d, float F, float *out) const {
        float t[ND];
#pragma unroll
        for (int k = 0; k < ND; k++) t[k] = d[k] * F - cs[k];
#pragma unroll
        for (int i = 0; i < ND; i++) {
            float v = 0.f;
#pragma unroll
            for (int j = 0; j < ND; j++) v = fmaf(m[i * ND + j], t[j], v);
            out[i] = v;
        }
    }
};

inline int phys_class(const DevCfg &c) {
    const bool anti = !(c.flags & SPHDEM_F_NO_ANTICLUMPING);
    if (!anti && c.visc == SPHDEM_VISC_MORRIS && c.var_h()) return PHYS_MORRIS_VARH;
    if (!anti && c.visc == SPHDEM_VISC_ARTIFICIAL && !c.var_h()) return PHYS_ARTIFICIAL;
    return PHYS_GENERIC;
}

template <int ND, int PHYS, bool TILE>
__global__ void __launch_bounds__(BLK) k_force(DevCfg c, const DevCfg *__restrict__ cp, DevState s, DevGlobals *__restrict__ g,
                                               const float4 *__restrict__ P0, const float4 *__restrict__ P1,
                                               const float4 *__restrict__ P2, float *__restrict__ om32,
                                               const int *__restrict__ tg, const int *__restrict__ nbr,
                                               const int *__restrict__ ncnt, int64_t ld, int64_t n,
                                               const float4 *__restrict__ NB, const double *__restrict__ cgrows,
                                               const int *__restrict__ start, const int *__restrict__ skey) {
    constexpr bool CG = PHYS == PHYS_CG;
    const float4 *shift = stencil_shifts(c, g);
    extern __shared__ float4 st_smem[];
    Staged st = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false};
    if constexpr (TILE) {
        const int n_t = start[g->n_sph_cells];
        const int64_t a0 = blockIdx.x * (int64_t)blockDim.x;
        if (a0 >= n_t) return;  /* no list owner in this block */
        st = stage_neighbours<ND, 3>(c, g, start, skey, P0, P1, P2, a0, n_t, st_smem);
        if (!st.ok) return;
    }
    const int visc = PHYS == PHYS_MORRIS_VARH ? SPHDEM_VISC_MORRIS
                     : (PHYS == PHYS_ARTIFICIAL ? SPHDEM_VISC_ARTIFICIAL : c.visc);
    const bool var_h = PHYS == PHYS_MORRIS_VARH ? true : (PHYS == PHYS_ARTIFICIAL ? false : c.var_h());
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float ndt = FLT_MAX;
    const int ta = a < n ? (tg[a] & 0xff) : -1;
    if (is_sph_or_sphb(ta)) {
        const float wcon = (float)c.wcon;
        const float4 pa = P0[a], va = P1[a], xa = P2[a];
        const float ha = pa.w, iha = xa.w;
        const float ihn2a = powi<ND>(iha) * iha * iha;
        const float densa = xa.x, pdr2a = xa.y, ma = va.w;
        /* VAR_H_CORRECTION: every gradient of a's sums carries 1/Omega_a
         * (gA = ga/Omega_a, gB = gb/Omega_a), so Omega_a (calcOmega,
         * sph.h:438-451) is summed in this same loop and the gradient sums
         * are scaled once at the end */
        const float ihna = powi<ND>(iha), pd_coef = ND * ihna * iha;
        Plain om;
        om.init(-ma * pd_coef * wK32(0.f, wcon));
        const bool sph = ta == T_SPH;
        const bool anti = PHYS == PHYS_GENERIC && !(c.flags & SPHDEM_F_NO_ANTICLUMPING);
        const float visc_nu = (float)c.viscosity, c0 = (float)c.spsound;
        const float liq_visc = (float)(2.0 * c.viscosity * c.dens);
        const float alpha_mon = (float)c.alpha_mon, alpha_art = (float)c.alpha_art;
        const float vdc = visc == SPHDEM_VISC_MONAGHAN ? 0.06f : 0.125f;
        const float k_anti_inv = c.k_anti != 0 ? (float)(1.0 / c.k_anti) : 0.f;
        Cg32<ND> cgw;
        if constexpr (CG) cgw.load(cgrows, s.cap, a);
        Kahan fp[ND], fv[ND], fb[ND], fa[ND];
        Kahan fq;  /* anticlumping: the same term on every component, not scaled by 1/Omega */
        fq.init(0.f);
#pragma unroll
        for (int k = 0; k < ND; k++) {
            fp[k].init(0.f);
            fv[k].init(0.f);
            fb[k].init(0.f);
            fa[k].init(0.f);
        }
        float hmin = FLT_MAX; /* smallest hav of the fluid pairs */
        const int cnt = ncnt[a];
        /* 8 entries at a time from the particle's list tiles (two int4 loads) */
        const int4 *tile = reinterpret_cast<const int4 *>(nbr + nl_at(a, 0, ld));
        int4 q0 = make_int4(-1, -1, -1, -1), q1 = q0;
#pragma unroll 2
        for (int j = 0; j < cnt; j++) {
            if ((j & 7) == 0) {
                q0 = __ldg(tile + (j >> 3) * 64);
                q1 = __ldg(tile + (j >> 3) * 64 + 1);
            }
            const int e = q0.x;
            q0 = make_int4(q0.y, q0.z, q0.w, q1.x);
            q1 = make_int4(q1.y, q1.z, q1.w, -1);
            if (e < 0) continue;
            const int b = e & B_MASK;
            float4 pb, vb, xb;
            if constexpr (TILE) {
                const int sl = st_slot<ND>(e >> B_BITS);
                const int off = b - st.lo[sl];
                if ((unsigned)off < (unsigned)st.num[sl]) {
                    const int k = st.base[sl] + off;
                    pb = st.S0[k];
                    vb = st.S1[k];
                    xb = st.S2[k];
                } else {
                    pb = P0[b];
                    vb = P1[b];
                    xb = P2[b];
                }
            } else {
                pb = P0[b];
                vb = P1[b];
                xb = P2[b];
            }
            /* sph / sphBoundary unless the packed mass is negative */
            const int tb = vb.w < 0.f ? (tg[b] & 0xff) : T_SPH;
            float d[3];
            nb_delta_t<ND>(e, shift, pa, pb, d);
            const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
            const float r = r2 * rinv;
            const float hb = pb.w, ihb = xb.w;
            const float ihn2b = powi<ND>(ihb) * ihb * ihb;
            const float qa = r * iha, qb = r * ihb;
            /* gradW: dr*F(q,h), F = ihn2*dK/dq/q, 1/q = h/r */
            const float Fa = qa != 0.f ? ihn2a * wdK32(qa, wcon) * (ha * rinv) : 0.f;
            const float Fb = qb != 0.f ? ihn2b * wdK32(qb, wcon) * (hb * rinv) : 0.f;
            float cA, cB, cM;  /* gA = d*cA, gB = d*cB, 0.5(gA+gB) = d*cM (times Omega_a with VAR_H) */
            if (var_h) {
                cA = Fa;
                cB = Fb;
                cM = 0.5f * (cA + cB);
                if (is_sph_or_sphb(tb)) om.add(vb.w * (ihna * (-qa * wdK32(qa, wcon) * iha) - pd_coef * wK32(qa, wcon)));
            } else {
                cA = cB = cM = 0.5f * (Fa + Fb);
            }
            /* corrected gradients: vectors gA, gB and their mean (times Omega_a with VAR_H) */
            float gAv[3] = {0.f, 0.f, 0.f}, gBv[3] = {0.f, 0.f, 0.f}, gMv[3] = {0.f, 0.f, 0.f};
            if constexpr (CG) {
                float wa[ND], wb[ND];
                cgw.apply(d, Fa, wa);
                cgw.apply(d, Fb, wb);
#pragma unroll
                for (int k = 0; k < ND; k++) {
                    gAv[k] = var_h ? wa[k] : 0.5f * (wa[k] + wb[k]);
                    gBv[k] = var_h ? wb[k] : 0.5f * (wa[k] + wb[k]);
                    gMv[k] = 0.5f * (gAv[k] + gBv[k]);
                }
            }
            const float densb = xb.x, mb = fabsf(vb.w);
            const float hav = 0.5f * (ha + hb);
            const float dv0 = va.x - vb.x, dv1 = va.y - vb.y, dv2 = va.z - vb.z;
            if (sph && tb != T_DEM && tb != T_DEMB) {
                const float vdr = d[0] * dv0 + d[1] * dv1 + d[2] * dv2;
                float vsig = 0.f;
                if (visc == SPHDEM_VISC_MORRIS) {
                    /* mb visc dg / (r^2 + 0.01 hav^2) with visc = num / (rho_a rho_b):
                     * one division, by the fast reciprocal (2 ulp) */
                    const float num = c.liq_dem() ? liq_visc : visc_nu * (densa + densb);
                    const float dg = CG ? d[0] * gMv[0] + d[1] * gMv[1] + d[2] * gMv[2] : r2 * cM;
                    const float sc = __fdividef(mb * num * dg, (densa * densb) * (r2 + 0.01f * hav * hav));
                    const float dvv[3] = {dv0, dv1, dv2};
#pragma unroll
                    for (int k = 0; k < ND; k++) fv[k].add(dvv[k] * sc);
                } else if (visc == SPHDEM_VISC_MONAGHAN) {
                    const float viss = vdr * rinv;
                    if (!c.liq_dem()) vsig = 2.f * c0 + 2.f * fabsf(viss);
                    const float sv = mb * (viss * vsig * alpha_mon / (densa + densb));
                    const float sc = sv * cM;
#pragma unroll
                    for (int k = 0; k < ND; k++) fv[k].add(CG ? sv * gMv[k] : sc * d[k]);
                } else if (visc == SPHDEM_VISC_ARTIFICIAL) {
                    if (vdr < 0.f) {
                        const float viss = vdr * rinv;
                        const float avsig = 2.f * c0 - 4.f * viss;
                        const float sv = mb * (viss * avsig * alpha_art / (densa + densb));
                        const float sc = sv * cM;
#pragma unroll
                        for (int k = 0; k < ND; k++) fa[k].add(CG ? sv * gMv[k] : sc * d[k]);
                        vsig = fmaxf(vsig, avsig);
                    }
                }
                /* the viscous bound vdc hav^2 / nu increases with hav, and so
                 * does the Courant bound 0.6 hav / vsig under Morris viscosity
                 * (vsig = 2 c0 for every pair): the loop's smallest hav gives
                 * them, bit for bit */
                hmin = fminf(hmin, hav);
                if (visc != SPHDEM_VISC_MORRIS) ndt = fminf(ndt, 0.6f * hav / vsig);
            }
            if (is_boundary(tb)) {
                float fbx[3] = {0.f, 0.f, 0.f};
                boundary32<ND>(cp, NB, b, d[0], d[1], d[2], r, dv0, dv1, dv2, ma, mb, fbx);
#pragma unroll
                for (int k = 0; k < ND; k++) fb[k].add(fbx[k]);
            } else if (tb == T_SPH || tb == T_SPHB) {
                const float pdr2b = xb.y;
                float antic = 0.f;
                if (anti) {
                    const float kdw = wK32(r / hav, wcon) * k_anti_inv;
                    antic = 0.01f * fabsf(pdr2a + pdr2b) * (kdw * kdw) * (kdw * kdw);
                }
                const float pc = pdr2a * cA + pdr2b * cB;
#pragma unroll
                for (int k = 0; k < ND; k++)
                    fp[k].add(CG ? -mb * (pdr2a * gAv[k] + pdr2b * gBv[k]) : -mb * (pc * d[k]));
                if (anti) fq.add(-mb * antic);
            }
        }
        if (hmin < FLT_MAX) {
            if (visc == SPHDEM_VISC_MORRIS) {
                const float vsig = 2.f * c0;
                ndt = fminf(ndt, 0.6f * hmin / vsig);
            }
            ndt = fminf(ndt, vdc * hmin * hmin / visc_nu);
        }
        float roma = 1.f;
        if (var_h) {
            /* Omega = 1 + h*sum/(rho*NDIM): an O(1) number, FP32 is ample */
            const float omega = 1.f + ha * om.s / (densa * ND);
            s.row(FD_OMEGA)[a] = omega;
            om32[a] = omega;
            roma = 1.f / omega;
        }
        float fsum2 = 0.f;
#pragma unroll
        for (int k = 0; k < ND; k++) {
            const float fpk = fp[k].s * roma + fq.s, fvk = fv[k].s * roma, fak = fa[k].s * roma;
            s.row(FD_FP + k)[a] += fpk;
            s.row(FD_FV + k)[a] += fvk;
            s.row(FD_FB + k)[a] += fb[k].s;
            double *f = s.row(FD_F + k);
            const double fk = f[a] + (double)((fak + fvk) + (fb[k].s + fpk));
            f[a] = fk;
            const float fkf = (float)fk;
            fsum2 += fkf * fkf;
        }
        /* accelCondition (sph.h:566-568), a dt bound: FP32 */
        ndt = fminf(ndt, 0.25f * sqrtf(ha * rsqrtf(fsum2)));
    }
    block_min_atomic(ndt, &g->new_dt_bits);
}

/* VH: VAR_H_CORRECTION known at compile time (1 on, 0 off) or read from
 * the configuration (-1) */
template <int ND, bool CG, int VH, bool TILE>
__global__ void __launch_bounds__(BLK) k_dddt(DevCfg c, DevState s, const DevGlobals *__restrict__ g,
                                              const float4 *__restrict__ P0, const float4 *__restrict__ P1,
                                              const float4 *__restrict__ P2, float *__restrict__ om32,
                                              const int *__restrict__ tg, const int *__restrict__ nbr,
                                              const int *__restrict__ ncnt, int64_t ld, int64_t n,
                                              const double *__restrict__ cgrows,
                                              const int *__restrict__ start, const int *__restrict__ skey) {
    const float4 *shift = stencil_shifts(c, g);
    const bool var_h = VH < 0 ? c.var_h() : VH == 1;
    extern __shared__ float4 st_smem[];
    Staged st = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false};
    if constexpr (TILE) {
        const int n_t = start[g->n_sph_cells];
        const int64_t a0 = blockIdx.x * (int64_t)blockDim.x;
        if (a0 >= n_t) return;  /* no list owner in this block */
        st = stage_neighbours<ND, 2>(c, const_cast<DevGlobals *>(g), start, skey, P0, P1, P2, a0, n_t, st_smem);
        if (!st.ok) return;
    }
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    const float wcon = (float)c.wcon;
    const float4 pa = P0[a], va = P1[a];
    const float ha = pa.w, iha = P2[a].w;
    const float ihn2a = powi<ND>(iha) * iha * iha;
    /* VAR_H_CORRECTION: the continuity sum carries 1/Omega_a only, so
     * Omega_a is summed in this loop and applied once at the end */
    const float ihna = powi<ND>(iha), pd_coef = ND * ihna * iha;
    Plain om;
    om.init(-va.w * pd_coef * wK32(0.f, wcon));
    Kahan acc;
    acc.init(0.f);
    Cg32<ND> cgw;
    if constexpr (CG) cgw.load(cgrows, s.cap, a);
    const int cnt = ncnt[a];
    /* 8 entries at a time from the particle's list tiles (two int4 loads) */
    const int4 *tile = reinterpret_cast<const int4 *>(nbr + nl_at(a, 0, ld));
    int4 q0 = make_int4(-1, -1, -1, -1), q1 = q0;
#pragma unroll 2
    for (int j = 0; j < cnt; j++) {
        if ((j & 7) == 0) {
            q0 = __ldg(tile + (j >> 3) * 64);
            q1 = __ldg(tile + (j >> 3) * 64 + 1);
        }
        const int e = q0.x;
        q0 = make_int4(q0.y, q0.z, q0.w, q1.x);
        q1 = make_int4(q1.y, q1.z, q1.w, -1);
        if (e < 0) continue;
        const int b = e & B_MASK;
        float4 pb, vb;
        if constexpr (TILE) {
            const int sl = st_slot<ND>(e >> B_BITS);
            const int off = b - st.lo[sl];
            if ((unsigned)off < (unsigned)st.num[sl]) {
                pb = st.S0[st.base[sl] + off];
                vb = st.S1[st.base[sl] + off];
            } else {
                pb = P0[b];
                vb = P1[b];
            }
        } else {
            pb = P0[b];
            vb = P1[b];
        }
        /* sph / sphBoundary unless the packed mass is negative */
        const int tb = vb.w < 0.f ? (tg[b] & 0xff) : T_SPH;
        const float mb = fabsf(vb.w);
        float d[3];
        nb_delta_t<ND>(e, shift, pa, pb, d);
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
        const float r = r2 * rinv;
        const float qa = r * iha;
        const float Fa = qa != 0.f ? ihn2a * wdK32(qa, wcon) * (ha * rinv) : 0.f;
        float F, Fb = 0.f;
        if (var_h) {
            F = Fa;
            if (is_sph_or_sphb(tb)) om.add(mb * (ihna * (-qa * wdK32(qa, wcon) * iha) - pd_coef * wK32(qa, wcon)));
        } else {
            const float ihb = P2[b].w;
            const float qb = r * ihb;
            Fb = qb != 0.f ? powi<ND>(ihb) * ihb * ihb * wdK32(qb, wcon) * (pb.w * rinv) : 0.f;
            F = 0.5f * (Fa + Fb);
        }
        const float dv[3] = {va.x - vb.x, va.y - vb.y, va.z - vb.z};
        float vdr;
        if constexpr (CG) {
            /* corrected gradient of a (and of b's kernel) applied with a's invM */
            float wa[ND], wb[ND];
            cgw.apply(d, Fa, wa);
            if (!var_h) cgw.apply(d, Fb, wb);
            vdr = 0.f;
#pragma unroll
            for (int k = 0; k < ND; k++) vdr += dv[k] * (var_h ? wa[k] : 0.5f * (wa[k] + wb[k]));
            F = 1.f;
        } else {
            vdr = dv[0] * d[0] + dv[1] * d[1] + dv[2] * d[2];
        }
        if (!(is_boundary(tb) || tb == T_DEM)) acc.add(mb * vdr * F);
    }
    float roma = 1.f;
    if (var_h) {
        const float omega = 1.f + ha * om.s / (P2[a].x * ND);
        s.row(FD_OMEGA)[a] = omega;
        om32[a] = omega;
        roma = 1.f / omega;
    }
    s.row(FD_DDDT)[a] += (double)(acc.s * roma);
}

/* ---------------------------------------------------------------------- */
/* SPH <-> DEM coupling sums over the reference's coupling neighbours
 * (calcNeighboursCoupling, dataLL.cpp:1104-1192: DEM within Rc, with the
 * asymmetric bucket rule).  MODE 0: calcPorosity + the DEM Shepard sums
 * (sph.h calcPorosity / calcShepSum); MODE 1: calcDEMtoSPHDrag +
 * finalisePorosity.
 *
 * Work split as in k_nlist: a warp takes 32 consecutive particles of the
 * bucket order, forms runs of buckets along the last axis, and stages the DEM
 * particles of every DEM bucket within Rc of the run in shared memory
 * (position in the run's frame, reference DEM bucket of the image, the
 * partner's packed fields); every lane then tests all staged partners.  The
 * Shepard contribution of one partner is reduced over the warp and added
 * with one FP64 atomic. */
constexpr int CP_WARPS = 8;
constexpr int CP_CAP = 128;

/* coupling_rule on packed bucket indices; lim_ceil = ceil(couple_lim), so
 * that for the integer sums rP < couple_lim <=> rP < lim_ceil */
template <int ND>
__device__ __forceinline__ bool coupling_rule_packed(int cs, int cd, int num, int lim_ceil) {
    int rP = 0, rM = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const int o = ((cd >> (10 * d)) & 1023) - ((cs >> (10 * d)) & 1023);
        if (o < -num || o > num) return false;
        rP += (o + 1) * (o + 1);
        rM += (o - 1) * (o - 1);
    }
    if (ND == 1) return true;
    return rP < lim_ceil || rM < lim_ceil;
}

/* one warp-aggregated atomic reserves k entries per lane of cnt; every lane
 * of the warp calls it; returns this lane's first entry */
__device__ __forceinline__ int64_t tap_reserve(int k, int *cnt) {
    const int lane = threadIdx.x & 31;
    int incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(cnt, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return (int64_t)base + incl - k;
}

/* TAP (adjoint replay only): the coupling pairs each fluid particle takes
 * go to the tap table tt of step *tslot -- mode 0 counts them and reserves
 * the particle's entries, mode 1 (same pairs, same order) writes them. */
template <int ND, int MODE, bool TAP>
__global__ void __launch_bounds__(CP_WARPS * 32, 3) k_couple(DevCfg c, const DevCfg *__restrict__ cp, DevState s,
                                                          const int *__restrict__ start, const int *__restrict__ skey,
                                                          const DevGlobals *__restrict__ g,
                                                          const float4 *__restrict__ P0, const float4 *__restrict__ P1,
                                                          const float4 *__restrict__ P2, const float4 *__restrict__ DP,
                                                          const int *__restrict__ tg, const int4 *__restrict__ RC4,
                                                          const int4 *__restrict__ win, int win_cap,
                                                          float *__restrict__ shep32, TapTable tt,
                                                          const int *__restrict__ tslot, int64_t n_all) {
    constexpr int Z = ND - 1;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ float4 s_pos[CP_WARPS][CP_CAP];
    __shared__ float4 s_aux[CP_WARPS][CP_CAP];
    __shared__ int2 s_id[CP_WARPS][CP_CAP];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    float4 *cpos = s_pos[w];
    float4 *caux = s_aux[w];
    int2 *cid = s_id[w];
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nsc = g->n_sph_cells;
    const int n_t = start[nsc];
    const int sdims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    const int zdim = sdims[Z];
    float cell[3];
    load_cell32(c, g, cell);
    const float cz = cell[Z];
    const float wcon = (float)c.wcon, two_over_rc = (float)c.two_over_rc;
    const float c_ihn = (float)c.c_ihn, c_ihn2 = (float)c.c_ihn2;
    const float por_incr = (float)c.por_incr, dem_vol = (float)c.dem_vol;
    const float rc2 = (float)c.rc2;
    const float rdens2d = (float)(1.0 / (2.0 * c.dem_radius));
    const int lim_ceil = (int)ceil(c.couple_lim);
    const float rc2x = (float)(2.0 * c.rc);
    const float rc_w = (float)c.rc * (1.f + 1e-5f);
    float dcf[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < ND; d++) dcf[d] = (float)c.dcell[d];

    for (int t0 = (blockIdx.x * CP_WARPS + w) * 32; t0 < n_t; t0 += CP_WARPS * gridDim.x * 32) {
        const int a = t0 + lane;
        int ta = -1, key = 0;
        if (a < n_t) {
            key = skey[a];
            ta = tg[a] & 0xff;
        }
        const bool act = is_sph_or_sphb(ta);
        if (MODE == 1 && is_boundary(ta)) s.row(FD_POR)[a] = 1.0;
        int ntap = 0, tag_a = 0, tlim = 0, js = 0;
        int *tout = nullptr;
        if (TAP) {
            js = *tslot;
            if (act) tag_a = s.irow(FI_TAG)[a];
            if (MODE == 1 && act) {
                const int2 o = tt.oc[(int64_t)js * n_all + tag_a];
                tout = tt.nb + (int64_t)js * tt.cap + o.x;
                tlim = o.y;
            }
        }
        int cc[3] = {0, 0, 0};
        decode<ND>(key, sdims, cc);
        const int col = key / zdim;
        /* this lane's particle: packed fields and reference DEM bucket */
        float4 pa0 = make_float4(0.f, 0.f, 0.f, 0.f), va = make_float4(0.f, 0.f, 0.f, 0.f);
        float dvol = 0.f, rdens = 0.f;
        int cs = 0;
        if (act) {
            pa0 = P0[a];
            va = P1[a];
            cs = RC4[a].x;
            const float densa = P2[a].x;
            dvol = va.w / densa;
            rdens = ND == 2 ? rdens2d / densa : 1.f / densa;
        }
        Kahan por, dpd, acc[ND];
        por.init(0.f);
        dpd.init(0.f);
#pragma unroll
        for (int k = 0; k < ND; k++) acc[k].init(0.f);

        unsigned pending = __ballot_sync(FULL, act);
        while (pending) {
            const int leader = __ffs(pending) - 1;
            const int lcol = __shfl_sync(FULL, col, leader);
            const int zmin = __shfl_sync(FULL, cc[Z], leader);
            const unsigned gmask = __ballot_sync(FULL, act && col == lcol && cc[Z] <= zmin + 2) & pending;
            pending &= ~gmask;
            const int zmax = __shfl_sync(FULL, cc[Z], 31 - __clz(gmask));
            int ccol[3] = {0, 0, 0};
#pragma unroll
            for (int d = 0; d < ND; d++) ccol[d] = __shfl_sync(FULL, cc[d], leader);
            const bool mine = (gmask >> lane) & 1u;
            float pv[3] = {1e30f, 1e30f, 1e30f};
            if (mine) {
                pv[0] = pa0.x;
                pv[1] = pa0.y;
                pv[2] = pa0.z;
                pv[Z] += (float)(cc[Z] - zmin) * cz;
            }
            /* DEM buckets within Rc of the run; the origin of DEM bucket k in
             * the run's frame (origin of bucket (ccol, zmin)) is
             * obase - (k - klo) * dcell, one FP64 difference per axis */
            int klo[3] = {0, 0, 0}, khi[3] = {0, 0, 0};
            float obase[3] = {0.f, 0.f, 0.f};
            float lmax = 0.f;
#pragma unroll
            for (int d = 0; d < ND; d++) {
                const int4 wlo = win[d * win_cap + (d == Z ? zmin : ccol[d])];
                klo[d] = wlo.x;
                khi[d] = d == Z ? win[d * win_cap + zmax].y : wlo.y;
                obase[d] = __int_as_float(wlo.z);
                if (c.periodic[d] && khi[d] - klo[d] + 1 > c.ddims[d]) khi[d] = klo[d] + c.ddims[d] - 1;
                lmax = fmaxf(lmax, (d == Z ? (float)(zmax - zmin + 1) : 1.f) * cell[d] + rc2x + 2.f * dcf[d]);
            }
            const float band_c = fp32_band(rc2, lmax * lmax);
            /* the run's extent on the last axis, widened by Rc and a rounding
             * margin: no DEM partner lies outside */
            float zw_lo = mine ? pv[Z] : 1e30f, zw_hi = mine ? pv[Z] : -1e30f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                zw_lo = fminf(zw_lo, __shfl_xor_sync(FULL, zw_lo, o));
                zw_hi = fmaxf(zw_hi, __shfl_xor_sync(FULL, zw_hi, o));
            }
            zw_lo -= rc_w + 1e-5f * lmax;
            zw_hi += rc_w + 1e-5f * lmax;
            int nst = 0;

            auto evaluate = [&]() {
                __syncwarp();
                for (int j = 0; j < nst; j++) {
                    const float4 q = cpos[j];
                    const float dd0 = pv[0] - q.x;
                    const float dd1 = ND > 1 ? pv[1] - q.y : 0.f;
                    const float dd2 = ND > 2 ? pv[2] - q.z : 0.f;
                    const float r2 = fmaf(dd2, dd2, fmaf(dd1, dd1, dd0 * dd0));
                    float wgt = 0.f;
                    if (r2 < rc2 + band_c) {
                        const int2 id = cid[j];
                        bool in = coupling_rule_packed<ND>(cs, id.y, c.couple_num, lim_ceil);
                        if (in && r2 >= rc2 - band_c) {
                            const int shp = (unsigned)id.x >> B_BITS;
                            in = exact_pair<ND>(cp, s, a, id.x & B_MASK, (shp & 3) - 1, ((shp >> 2) & 3) - 1,
                                                ((shp >> 4) & 3) - 1, c.rc2, 1);
                        }
                        if (in) {
                            if (TAP) {
                                if (MODE == 1 && ntap < tlim) tout[ntap] = s.irow(FI_TAG)[id.x & B_MASK] | (id.x & ~B_MASK);
                                ntap++;
                            }
                            const float r = sqrtf(r2);
                            const float qq = r * two_over_rc;
                            wgt = c_ihn * wK32(qq, wcon);
                            const float4 x = caux[j];
                            if (MODE == 0) {
                                por.add(por_incr * wgt);
                                if (r != 0.f) {
                                    const float Fq = c_ihn2 * wdK32(qq, wcon) / qq;
                                    const float vd = (va.x - x.x) * dd0 + (va.y - x.y) * dd1 + (va.z - x.z) * dd2;
                                    dpd.add(-dem_vol * vd * Fq);
                                    const float ddv[3] = {dd0, dd1, dd2};
#pragma unroll
                                    for (int k = 0; k < ND; k++) acc[k].add(dem_vol * ddv[k] * Fq);
                                }
                            } else {
                                /* x = (m/shep, fdrag) of the DEM particle */
                                const float sc = x.x * rdens * wgt;
                                const float fdb[3] = {x.y, x.z, x.w};
#pragma unroll
                                for (int k = 0; k < ND; k++) acc[k].add(-sc * fdb[k]);
                            }
                        }
                    }
                    if (MODE == 0 && __any_sync(FULL, wgt != 0.f)) {
                        const float sum = warp_sum(dvol * wgt);
                        if (lane == 0 && sum != 0.f) atomicAdd(&shep32[cid[j].x & B_MASK], sum);
                    }
                }
                __syncwarp();
                nst = 0;
            };

            /* Range table in rounds of 32 lanes: one lane per (DEM column of the
             * window, period piece along the last axis), each a run of
             * consecutive DEM keys.  All lanes load their ranges at once; the
             * candidates of a round are then gathered flat. */
            int nwcol = 1;
#pragma unroll
            for (int d = 0; d < Z; d++) nwcol *= khi[d] - klo[d] + 1;
            const int nranges = 3 * nwcol;
            const int ddz = c.ddims[Z];
            const int dstart = nsc;
            int r0 = -32, t = 0, total = 0;
            int r_b0 = 0, r_cnt = 0, r_lin = 0, r_zq = 0, r_sh = 0, r_excl = 0;
            float r_dx = 0.f, r_dy = 0.f;
            /* next round of ranges with at least one candidate */
            auto load_round = [&]() -> bool {
                for (r0 += 32; r0 < nranges; r0 += 32) {
                    r_b0 = r_cnt = r_lin = r_zq = r_sh = 0;
                    r_dx = r_dy = 0.f;
                    const int ri = r0 + lane;
                    if (ri < nranges) {
                        const int colq = ri / 3, wz = ri % 3 - 1;
                        int kq[2] = {0, 0};
                        if (Z == 2) {
                            const int nwy = khi[1] - klo[1] + 1;
                            kq[0] = klo[0] + colq / nwy;
                            kq[1] = klo[1] + colq % nwy;
                        } else if (Z == 1) {
                            kq[0] = klo[0] + colq;
                        }
                        int col_lin = 0, shp = 0;
                        float dl[2] = {0.f, 0.f};
#pragma unroll
                        for (int d = ND; d < 3; d++) shp |= 1 << (2 * d);
#pragma unroll
                        for (int d = 0; d < Z; d++) {
                            int tt = kq[d], shd = 0;
                            if (tt < 0) {
                                tt += c.ddims[d];
                                shd = -1;
                            } else if (tt >= c.ddims[d]) {
                                tt -= c.ddims[d];
                                shd = 1;
                            }
                            col_lin = col_lin * c.ddims[d] + tt;
                            dl[d] = (float)(kq[d] - klo[d]) * dcf[d] - obase[d];
                            shp |= (shd + 1) << (2 * d);
                        }
                        shp |= (wz + 1) << (2 * Z);
                        const bool ok = wz == 0 || c.periodic[Z];
                        const int zlo = max(klo[Z], wz * ddz), zhi = min(khi[Z], (wz + 1) * ddz - 1);
                        if (ok && zlo <= zhi) {
                            r_lin = dstart + col_lin * ddz + (zlo - wz * ddz);
                            r_b0 = start[r_lin];
                            r_cnt = start[r_lin + (zhi - zlo) + 1] - r_b0;
                            r_zq = zlo - klo[Z];
                            r_sh = shp;
                            r_dx = dl[0];
                            r_dy = dl[1];
                            /* DEM buckets hold their particles sorted on the last axis:
                             * keep those within Rc of the run there (binary search) */
                            int lo = 0, hi = r_cnt;
                            while (lo < hi) {
                                const int mid = (lo + hi) >> 1, b = r_b0 + mid;
                                const float4 q = P0[b];
                                const float z = (Z == 0 ? q.x : (Z == 1 ? q.y : q.z)) +
                                                ((float)(r_zq + skey[b] - r_lin) * dcf[Z] - obase[Z]);
                                if (z < zw_lo) lo = mid + 1;
                                else hi = mid;
                            }
                            const int first = lo;
                            hi = r_cnt;
                            while (lo < hi) {
                                const int mid = (lo + hi) >> 1, b = r_b0 + mid;
                                const float4 q = P0[b];
                                const float z = (Z == 0 ? q.x : (Z == 1 ? q.y : q.z)) +
                                                ((float)(r_zq + skey[b] - r_lin) * dcf[Z] - obase[Z]);
                                if (z <= zw_hi) lo = mid + 1;
                                else hi = mid;
                            }
                            r_b0 += first;
                            r_cnt = lo - first;
                        }
                    }
                    r_excl = r_cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(FULL, r_excl, o);
                        if (lane >= o) r_excl += v;
                    }
                    total = __shfl_sync(FULL, r_excl, 31);
                    r_excl -= r_cnt;
                    t = 0;
                    if (total > 0) return true;
                }
                return false;
            };

            bool more = load_round();
            for (;;) {
                while (more && nst + 32 <= CP_CAP) {
                    const int j = t + lane;
                    int src = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int e = __shfl_sync(FULL, r_excl, src + step);
                        if (e <= j) src += step;
                    }
                    const int b0 = __shfl_sync(FULL, r_b0, src), ex = __shfl_sync(FULL, r_excl, src);
                    const int lin = __shfl_sync(FULL, r_lin, src), zq = __shfl_sync(FULL, r_zq, src);
                    const int shp = __shfl_sync(FULL, r_sh, src);
                    const float dx = __shfl_sync(FULL, r_dx, src), dy = __shfl_sync(FULL, r_dy, src);
                    bool valid = false;
                    float4 pb = make_float4(0.f, 0.f, 0.f, 0.f), xb = make_float4(0.f, 0.f, 0.f, 0.f);
                    int b = 0, cdp = 0;
                    float dzl = 0.f;
                    if (j < total) {
                        b = b0 + (j - ex);
                        const int tgb = tg[b];
                        const int shv[3] = {(shp & 3) - 1, ((shp >> 2) & 3) - 1, ((shp >> 4) & 3) - 1};
                        valid = (tgb & 0xff) == T_DEM && (shp == 0x15 || img_ok<ND>(tgb >> 8, shv));
                        if (valid) {
                            pb = P0[b];
                            xb = MODE == 0 ? P1[b] : DP[b];
                            dzl = (float)(zq + (skey[b] - lin)) * dcf[Z] - obase[Z];
                            const int4 rc = RC4[b];
                            cdp = rc.x;
#pragma unroll
                            for (int d = 0; d < ND; d++) {
                                const int m = 1023 << (10 * d);
                                if (shv[d]) cdp = (cdp & ~m) | ((shv[d] < 0 ? rc.y : rc.z) & m);
                            }
                        }
                    }
                    const unsigned m = __ballot_sync(FULL, valid);
                    if (valid) {
                        const int pos = nst + __popc(m & lt_mask);
                        float qv[3] = {pb.x, pb.y, pb.z};
                        if (Z > 0) qv[0] += dx;
                        if (Z > 1) qv[1] += dy;
                        qv[Z] += dzl;
                        cpos[pos] = make_float4(qv[0], qv[1], qv[2], 0.f);
                        caux[pos] = xb;
                        cid[pos] = make_int2(b | (shp << B_BITS), cdp);
                    }
                    nst += __popc(m);
                    t += 32;
                    if (t >= total) more = load_round();
                }
                evaluate();
                if (!more) break;
            }
        }
        if (TAP && MODE == 0) {
            const int64_t off = tap_reserve(ntap, tt.cnt + js);
            if (act) tt.oc[(int64_t)js * n_all + tag_a] = make_int2((int)off, off + ntap <= tt.cap ? ntap : 0);
        }
        if (!act) continue;
        if (MODE == 0) {
            s.row(FD_POR)[a] = por.s;
            s.row(FD_DPORDT)[a] = dpd.s;
#pragma unroll
            for (int k = 0; k < ND; k++) s.row(FD_GPOR + k)[a] = acc[k].s;
        } else {
#pragma unroll
            for (int k = 0; k < ND; k++) {
                const double v = acc[k].s;
                s.row(FD_FDRAG + k)[a] = v;
                s.row(FD_F + k)[a] += v;
            }
            double p = 1.0 - s.row(FD_POR)[a];
            if (p < 0.37) {
                p = 0.37;
                s.row(FD_DPORDT)[a] = 0.0;
                for (int k = 0; k < 3; k++) s.row(FD_GPOR + k)[a] = 0.0;
            }
            s.row(FD_POR)[a] = p;
        }
    }
}

/* (m/shep, fdrag) of every DEM particle for the DEM->SPH drag (sph.h:1359) */
__global__ void k_pack_dem_drag(DevState s, const float *__restrict__ shep32, const float4 *__restrict__ P1,
                                float4 *__restrict__ DP, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (s.irow(FI_IAM)[i] != T_DEM) return;
    /* the Shepard sum was accumulated in FP32 by k_couple<.., 0> */
    const float sh = shep32[i];
    s.row(FD_SHEP)[i] = sh;
    DP[i] = make_float4(sh != 0.f ? P1[i].w / sh : 0.f, (float)s.row(FD_FDRAG)[i], (float)s.row(FD_FDRAG + 1)[i],
                        (float)s.row(FD_FDRAG + 2)[i]);
}

/* One lane's entry of a bucket range table around a run of buckets (ccol
 * on the leading axes, zmin..zmax on the last axis Z): lane = 3 * column +
 * period piece, for the 3^(d-1) neighbour columns; each entry is a run of
 * consecutive keys key0 + lin .. (buckets zmin-1 .. zmax+1 of the column,
 * cut at a periodic seam).  Entries of other lanes are empty. */
struct RangeEntry {
    int b0, cnt, lin, zoff, shp, code;
    float ox, oy;
};

template <int ND>
__device__ __forceinline__ RangeEntry range_entry(int lane, const int *ccol, int zmin, int zmax, const int *dims,
                                                  const int *periodic, const float *cell, int key0,
                                                  const int *__restrict__ start) {
    constexpr int Z = ND - 1;
    constexpr int NCOL = Z == 2 ? 9 : (Z == 1 ? 3 : 1);
    RangeEntry r = {0, 0, 0, 0, 0x15, 0, 0.f, 0.f};
    if (lane >= 3 * NCOL) return r;
    const int colidx = lane / 3, wz = lane % 3 - 1;
    int o[2] = {0, 0};
    if (Z == 2) {
        o[0] = colidx / 3 - 1;
        o[1] = colidx % 3 - 1;
    } else if (Z == 1) {
        o[0] = colidx - 1;
    }
    bool ok = wz == 0 || periodic[Z];
    int col_lin = 0, code = 0, shp = 0;
    float off[2] = {0.f, 0.f};
#pragma unroll
    for (int d = ND; d < 3; d++) {
        shp |= 1 << (2 * d);
        code += code_stride(d);
    }
#pragma unroll
    for (int d = 0; d < Z; d++) {
        int t = ccol[d] + o[d], shd = 0;
        if (t < 0) {
            ok = ok && periodic[d];
            t += dims[d];
            shd = -1;
        } else if (t >= dims[d]) {
            ok = ok && periodic[d];
            t -= dims[d];
            shd = 1;
        }
        col_lin = col_lin * dims[d] + t;
        code += (o[d] + 1) * code_stride(d);
        off[d] = (float)o[d] * cell[d];
        shp |= (shd + 1) << (2 * d);
    }
    shp |= (wz + 1) << (2 * Z);
    const int zdim = dims[Z];
    const int zlo = max(zmin - 1, wz * zdim), zhi = min(zmax + 1, (wz + 1) * zdim - 1);
    if (ok && zlo <= zhi) {
        r.lin = key0 + col_lin * zdim + (zlo - wz * zdim);
        r.b0 = start[r.lin];
        r.cnt = start[r.lin + (zhi - zlo) + 1] - r.b0;
        r.zoff = zlo - zmin;
        r.shp = shp;
        r.code = code << B_BITS;
        r.ox = off[0];
        r.oy = off[1];
    }
    return r;
}

/* exclusive prefix of v over the warp; *total = the sum */
__device__ __forceinline__ int warp_excl_scan(int v, int lane, int *total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    *total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

/* the lane whose range holds flat index j: the last lane with excl <= j */
__device__ __forceinline__ int warp_range_src(int excl, int j) {
    int src = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int e = __shfl_sync(0xffffffffu, excl, src + step);
        if (e <= j) src += step;
    }
    return src;
}

/* One DEM-DEM contact in FP64 (calcDEMContacts, sph.h:1676-1706): the
 * overlap (Ra + Rb) - r cancels, so r and the spring-dashpot force are FP64 */
template <int ND>
__device__ __noinline__ bool dem_contact(const DevCfg *__restrict__ cp, const DevState s, int a, int b,
                                         const int *sh, double *fc) {
    const double Ra = s.row(FD_RADIUS)[a] > 0 ? s.row(FD_RADIUS)[a] : cp->dem_radius;
    const double Rb = s.row(FD_RADIUS)[b] > 0 ? s.row(FD_RADIUS)[b] : cp->dem_radius;
    double dx[3] = {0, 0, 0}, r = 0.0;
#pragma unroll
    for (int k = 0; k < ND; k++) {
        dx[k] = s.row(FD_R + k)[a] - image_pos(s.row(FD_R + k)[b], sh[k], cp->rmin[k], cp->rmax[k]);
        r += dx[k] * dx[k];
    }
    r = sqrt(r);
    const double overlap = (Ra + Rb) - r;
    if (!(overlap > 0.0)) return false;
    const double ma = s.row(FD_MASS)[a];
    double odot = 0.0;
#pragma unroll
    for (int k = 0; k < ND; k++) odot -= (s.row(FD_VHAT + k)[a] - s.row(FD_VHAT + k)[b]) * (dx[k] / r);
    const double sN = cp->dem_k * overlap + cp->dem_gamma * odot;
#pragma unroll
    for (int k = 0; k < ND; k++) fc[k] += (sN * (dx[k] / r)) / ma;
    return true;
}

/* TAP: a warp's passing candidates of one round go to the owner's fixed
 * slots (out, per of them) in lane order; every lane calls it once per
 * round of the warp-uniform candidate loop */
__device__ __forceinline__ void tap_flush(bool &hit, int &ent, int *out, int per, int &k) {
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    const int pos = k + __popc(m & ((1u << (threadIdx.x & 31)) - 1u));
    if (hit && out && pos < per) out[pos] = ent;
    k += __popc(m);
    hit = false;
}

/* Update of DEM particle a from its warp-reduced FPI and contact sums
 * (calcFPI normalisation, sph.h:1708-1792; Di Felice drag, sph.h:1575-1631,
 * with the drag coefficient in FP32); state accumulation in FP64 */
template <int ND>
__device__ __noinline__ void dem_end_update(const DevCfg *__restrict__ cp, const DevState s, int a, float sum,
                                            float por, const float *fpfb, const float *fv, const float *fvel,
                                            const double *fc) {
    double f[3] = {0, 0, 0}, fpv[3] = {0, 0, 0};
    float vel[3] = {0.f, 0.f, 0.f}, fdrag_out[3] = {0.f, 0.f, 0.f};
    float pr = por;
#pragma unroll
    for (int k = 0; k < ND; k++) {
        f[k] = s.row(FD_F + k)[a];
        fpv[k] = s.row(FD_FP + k)[a];
        vel[k] = fvel[k];
    }
    if (sum > 0.5f) {
        const float rsum = 1.f / sum;
        float fpfbd[3] = {0.f, 0.f, 0.f}, fvd[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < ND; k++) {
            fpfbd[k] = fpfb[k] * rsum;
            fvd[k] = fv[k] * rsum;
            vel[k] *= rsum;
            s.row(FD_FB + k)[a] = fpfbd[k];
            s.row(FD_FV + k)[a] = fvd[k];
        }
        pr *= rsum;
        float dv[3] = {0.f, 0.f, 0.f}, vd2 = 0.f;
#pragma unroll
        for (int k = 0; k < ND; k++) {
            dv[k] = pr * (vel[k] - (float)s.row(FD_VHAT + k)[a]);
            vd2 += dv[k] * dv[k];
        }
        const float vdiff = sqrtf(vd2);
        float fdv[3] = {0.f, 0.f, 0.f};
        if (vdiff != 0.f) {
            const float A = (float)(cp->pi * (cp->dem_radius * cp->dem_radius));
            const float Re = (float)(2.0 * cp->dem_radius / cp->viscosity) * vdiff;
            const float lg = 1.5f - log10f(Re);
            const float dragGamma = 3.7f - 0.65f * expf(-(lg * lg) / 2.f);
            const float cc0 = 0.63f + 4.8f / sqrtf(Re);
            const float sc = 0.5f * A * (cc0 * cc0) * vdiff;
            const float pw = powf(pr, -dragGamma) * (float)cp->drag_scale;
#pragma unroll
            for (int k = 0; k < ND; k++) fdv[k] = sc * dv[k] * pw;
        }
        const double ma = s.row(FD_MASS)[a];
        const float vm = (float)(cp->dem_vol / ma), dm = (float)(cp->dens / ma);
#pragma unroll
        for (int k = 0; k < ND; k++) {
            fdrag_out[k] = vm * (fvd[k] + fpfbd[k]) + dm * fdv[k];
            f[k] += fdrag_out[k];
        }
    }
    for (int k = 0; k < 3; k++) {
        s.row(FD_FVEL + k)[a] = vel[k];
        s.row(FD_FDRAG + k)[a] = fdrag_out[k];
    }
    s.row(FD_POR)[a] = pr;
    s.row(FD_SHEP)[a] = sum;
#pragma unroll
    for (int k = 0; k < ND; k++) {
        s.row(FD_F + k)[a] = f[k] + fc[k];
        s.row(FD_FP + k)[a] = fpv[k] + fc[k];
    }
}

/* ---------------------------------------------------------------------- */
/* calcFPI + calcParticleDrag + calcDEMContacts, one warp per DEM particle.
 * The candidates of the 3^d SPH buckets and of the 3^d DEM buckets come from
 * range tables (one lane per bucket run, all loaded at once) and are spread
 * flat over the lanes; sums are reduced over the warp.  Contacts (the overlap
 * 2R - r cancels) and the state update are FP64; the Di Felice drag
 * coefficient is FP32. */
/* TAP (adjoint replay only): the FPI partners and the contacts with positive
 * overlap of each DEM particle also go to the tap tables tf / tct of step
 * *tslot (DEM particle w of the DEM range owns slots w * per). */
template <int ND, bool TAP>
__global__ void __launch_bounds__(BLK) k_dem_end(DevCfg c, const DevCfg *__restrict__ cp, DevState s,
                                                 const int *__restrict__ start, const int *__restrict__ skey,
                                                 const DevGlobals *__restrict__ g, const float4 *__restrict__ P0,
                                                 const float4 *__restrict__ P1, const float4 *__restrict__ P2,
                                                 const float4 *__restrict__ Q0, const float4 *__restrict__ Q1,
                                                 const float4 *__restrict__ Q2, const int *__restrict__ tg,
                                                 const float4 *__restrict__ DS, TapTable tf, TapTable tct,
                                                 const int *__restrict__ tslot, int64_t n_all) {
    constexpr int Z = ND - 1;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int warps = (blockDim.x >> 5) * gridDim.x;
    const int nsc = g->n_sph_cells;
    const int dem0 = start[nsc], dem1 = start[nsc + c.n_dem_cells];
    const int sdims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    float cell[3], dcellf[3];
    load_cell32(c, g, cell);
    float cs2 = 0.f, cd2 = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        dcellf[d] = (float)c.dcell[d];
        if (d < ND) {
            cs2 = fmaxf(cs2, 4.f * cell[d] * cell[d]);
            cd2 = fmaxf(cd2, 4.f * dcellf[d] * dcellf[d]);
        }
    }
    const float wcon = (float)c.wcon;
    for (int a = dem0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); a < dem1; a += warps) {
        if ((tg[a] & 0xff) != T_DEM) continue;
        const float4 pa = P0[a];
        const float ha = pa.w;
        /* tap state: this lane's pending entry, entries so far, owner slots */
        bool thit = false;
        int tent = 0, kf = 0, kc = 0, js = 0;
        int *fout = nullptr, *cout = nullptr;
        if (TAP) {
            js = *tslot;
            const int64_t w = a - dem0;
            if ((w + 1) * tf.per <= tf.cap) fout = tf.nb + (int64_t)js * tf.cap + w * tf.per;
            if ((w + 1) * tct.per <= tct.cap) cout = tct.nb + (int64_t)js * tct.cap + w * tct.per;
        }
        /* FPI over the SPH candidates: this particle in its SPH bucket's frame */
        const float4 ds = DS[a];
        int cs[3] = {0, 0, 0};
        decode<ND>(__float_as_int(ds.w), sdims, cs);
        const float oa[3] = {ds.x, ds.y, ds.z};
        float sum = 0.f, por = 0.f;
        float fpfb[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, fvel[3] = {0, 0, 0};
        {
            const RangeEntry re = range_entry<ND>(lane, cs, cs[Z], cs[Z], sdims, c.periodic, cell, 0, start);
            int total = 0;
            const int excl = warp_excl_scan(re.cnt, lane, &total);
            for (int t = 0; t < total; t += 32) {
                if (TAP) tap_flush(thit, tent, fout, tf.per, kf);
                const int j = t + lane;
                const int src = warp_range_src(excl, j);
                const int b0 = __shfl_sync(FULL, re.b0, src), ex = __shfl_sync(FULL, excl, src);
                const int lin = __shfl_sync(FULL, re.lin, src), zoff = __shfl_sync(FULL, re.zoff, src);
                const int shp = __shfl_sync(FULL, re.shp, src);
                const float ox = __shfl_sync(FULL, re.ox, src), oy = __shfl_sync(FULL, re.oy, src);
                if (j >= total) continue;
                const int b = b0 + (j - ex);
                const float4 pb = P0[b];
                const int zrel = zoff + (skey[b] - lin);
                float qv[3] = {pb.x, pb.y, pb.z};
                if (Z > 0) qv[0] += ox;
                if (Z > 1) qv[1] += oy;
                qv[Z] += (float)zrel * cell[Z];
                const float d0 = oa[0] - qv[0];
                const float d1 = ND > 1 ? oa[1] - qv[1] : 0.f;
                const float d2 = ND > 2 ? oa[2] - qv[2] : 0.f;
                const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
                const float tt = 2.f * fmaxf(ha, pb.w);
                const float T = tt * tt;
                const float band = fp32_band(T, cs2);
                if (r2 > T + band) continue;
                const int sh[3] = {(shp & 3) - 1, ((shp >> 2) & 3) - 1, ((shp >> 4) & 3) - 1};
                if (r2 >= T - band && !exact_pair<ND>(cp, s, a, b, sh[0], sh[1], sh[2], 0.0, 0)) continue;
                const int tgb = tg[b];
                if (shp != 0x15 && !img_ok<ND>(tgb >> 8, sh)) continue;
                if ((tgb & 0xff) == T_BOUNDARY) continue;
                const float4 vb = P1[b], xb = P2[b];
                const float mb = fabsf(vb.w);
                const float q = sqrtf(r2) * xb.w;
                const float Wab = powi<ND>(xb.w) * wK32(q, wcon);
                const float dvW = (mb / xb.x) * Wab, mW = mb * Wab;
                const float4 q0 = Q0[b], q1 = Q1[b];
                const float fvb[3] = {q0.w, q1.x, q1.y};
                const float fb_[3] = {q0.x, q0.y, q0.z};
#pragma unroll
                for (int k = 0; k < ND; k++) {
                    fpfb[k] += mW * fb_[k];
                    fv[k] += mW * fvb[k] + dvW * fvb[k];
                }
                fvel[0] += dvW * vb.x;
                fvel[1] += dvW * vb.y;
                fvel[2] += dvW * vb.z;
                por += dvW * xb.z;
                sum += dvW;
                if (TAP) {
                    thit = true;
                    tent = s.irow(FI_TAG)[b] | (shp << B_BITS);
                }
            }
            if (TAP) tap_flush(thit, tent, fout, tf.per, kf);
        }
        sum = warp_sum(sum);
        por = warp_sum(por);
#pragma unroll
        for (int k = 0; k < ND; k++) {
            fpfb[k] = warp_sum(fpfb[k]);
            fv[k] = warp_sum(fv[k]);
            fvel[k] = warp_sum(fvel[k]);
        }
        /* DEM contacts over the DEM grid (sph.h:1676-1706), FP64 per contact */
        int cdm[3] = {0, 0, 0};
        decode<ND>(skey[a] - nsc, c.ddims, cdm);
        const float od[3] = {pa.x, pa.y, pa.z};
        const float Ra_f = P2[a].y;
        double fc[3] = {0, 0, 0};
        {
            const RangeEntry re = range_entry<ND>(lane, cdm, cdm[Z], cdm[Z], c.ddims, c.periodic, dcellf, nsc, start);
            int total = 0;
            const int excl = warp_excl_scan(re.cnt, lane, &total);
            for (int t = 0; t < total; t += 32) {
                if (TAP) tap_flush(thit, tent, cout, tct.per, kc);
                const int j = t + lane;
                const int src = warp_range_src(excl, j);
                const int b0 = __shfl_sync(FULL, re.b0, src), ex = __shfl_sync(FULL, excl, src);
                const int lin = __shfl_sync(FULL, re.lin, src), zoff = __shfl_sync(FULL, re.zoff, src);
                const int shp = __shfl_sync(FULL, re.shp, src);
                const float ox = __shfl_sync(FULL, re.ox, src), oy = __shfl_sync(FULL, re.oy, src);
                if (j >= total) continue;
                const int b = b0 + (j - ex);
                if (b == a && shp == 0x15) continue;
                const int tgb = tg[b];
                if ((tgb & 0xff) != T_DEM) continue;
                const float4 pb = P0[b];
                const int zrel = zoff + (skey[b] - lin);
                float qv[3] = {pb.x, pb.y, pb.z};
                if (Z > 0) qv[0] += ox;
                if (Z > 1) qv[1] += oy;
                qv[Z] += (float)zrel * dcellf[Z];
                const float d0 = od[0] - qv[0];
                const float d1 = ND > 1 ? od[1] - qv[1] : 0.f;
                const float d2 = ND > 2 ? od[2] - qv[2] : 0.f;
                const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
                const float tt = 2.f * fmaxf(ha, pb.w);
                const float T = tt * tt;
                const float band = fp32_band(T, cd2);
                if (r2 > T + band) continue;
                const int sh[3] = {(shp & 3) - 1, ((shp >> 2) & 3) - 1, ((shp >> 4) & 3) - 1};
                if (r2 >= T - band && !exact_pair<ND>(cp, s, a, b, sh[0], sh[1], sh[2], 0.0, 0)) continue;
                if (shp != 0x15 && !img_ok<ND>(tgb >> 8, sh)) continue;
                if ((Ra_f + P2[b].y) * 1.0001f - sqrtf(r2) <= 0.f) continue;
                const bool touch = dem_contact<ND>(cp, s, a, b, sh, fc);
                if (TAP && touch) {
                    thit = true;
                    tent = s.irow(FI_TAG)[b] | (shp << B_BITS);
                }
            }
            if (TAP) tap_flush(thit, tent, cout, tct.per, kc);
        }
        if (TAP && lane == 0) {
            const int64_t w = a - dem0, at = (int64_t)js * n_all + s.irow(FI_TAG)[a];
            tf.oc[at] = make_int2((int)(w * tf.per), fout && kf <= tf.per ? kf : 0);
            if (!fout || kf > tf.per) atomicMax(tf.cnt + js, (int)tf.cap + 1);   /* marks the step overflowed */
            tct.oc[at] = make_int2((int)(w * tct.per), cout && kc <= tct.per ? kc : 0);
            if (!cout || kc > tct.per) atomicMax(tct.cnt + js, (int)tct.cap + 1);
        }
#pragma unroll
        for (int k = 0; k < ND; k++)
            for (int oo = 16; oo > 0; oo >>= 1) fc[k] += __shfl_xor_sync(FULL, fc[k], oo);
        if (lane == 0) dem_end_update<ND>(cp, s, a, sum, por, fpfb, fv, fvel, fc);
    }
}

/* rows of the neighbour list in tag order (count pass when idx == nullptr) */
__global__ void k_list_export(DevState s, const int *tg, const int *nbr, const int *ncnt, int64_t ld, int64_t n,
                              int *cnt, const long long *offs, int *idx) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    const int tag = s.irow(FI_TAG)[a];
    const int m = ncnt[a];
    if (!idx) {
        int v = 0;
        for (int j = 0; j < m; j++) v += nbr[nl_at(a, j, ld)] >= 0;
        cnt[tag] = v;
        return;
    }
    int k = 0;
    for (int j = 0; j < m; j++) {
        const int e = nbr[nl_at(a, j, ld)];
        if (e >= 0) idx[offs[tag] + k++] = s.irow(FI_TAG)[e & B_MASK];
    }
}

/* The list rows of the SPH/SPHB particles as the adjoint's per-step pair
 * tables, in tag space: nb[slot * cap + off + k] = tag_b | shift << 26 (shift
 * = (sh_x + 1) | (sh_y + 1) << 2 | (sh_z + 1) << 4, the periodic image of b),
 * oc[slot * n + tag_a] = (off, count).  One atomic per warp reserves the
 * warp's entries; an overflowing particle records count 0 and the caller sees
 * cnt[slot] > cap. */
template <int ND>
__global__ void k_adj_pairs(DevState s, const DevGlobals *__restrict__ g, const int *__restrict__ skey,
                            const int *__restrict__ tg, const int *__restrict__ nbr, const int *__restrict__ ncnt,
                            int64_t ld, int64_t n, int *nb, int2 *oc, int *cnt, int64_t cap,
                            const int *__restrict__ slot) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = a < n && is_sph_or_sphb(tg[a] & 0xff);
    const int m = live ? ncnt[a] : 0;
    int k = 0;
    for (int j = 0; j < m; j++) k += nbr[nl_at(a, j, ld)] >= 0;
    const int lane = threadIdx.x & 31;
    int incl = k;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int js = *slot;
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(cnt + js, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!live) return;
    const int64_t off = (int64_t)base + incl - k;
    const int64_t room = cap - off;
    int *out = nb + (int64_t)js * cap + off;
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    int cc[3] = {0, 0, 0};
    decode<ND>(skey[a], dims, cc);
    int q = 0;
    for (int j = 0; j < m && q < room; j++) {
        const int e = nbr[nl_at(a, j, ld)];
        if (e < 0) continue;
        int o[3];
        nl_decode_code(e >> B_BITS, o);
        int code = 0;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            int sh = 0;
            if (d < ND) {
                const int t = cc[d] + o[d];
                sh = t < 0 ? -1 : (t >= dims[d] ? 1 : 0);
            }
            code |= (sh + 1) << (2 * d);
        }
        out[q++] = s.irow(FI_TAG)[e & B_MASK] | (code << B_BITS);
    }
    oc[(int64_t)js * n + s.irow(FI_TAG)[a]] = make_int2((int)off, room >= k ? k : 0);
}

int warp_blocks(int items) { return std::max(1, std::min(1 << 16, (items + (BLK / 32) - 1) / (BLK / 32))); }
/* coupling passes: grid-stride over 32-particle slices, one wave of resident blocks */
template <int ND, int MODE>
int resident_blocks(int64_t particles) {
    static int resident = 0;
    if (!resident) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_couple<ND, MODE, false>, CP_WARPS * 32, 0);
        resident = std::max(1, sms * per_sm);
    }
    const int64_t need = (particles + 32 * CP_WARPS - 1) / (32 * CP_WARPS);
    return (int)std::max<int64_t>(1, std::min<int64_t>(resident, need));
}

template <int ND>
int dem_end_blocks(int64_t particles) {
    static int resident = 0;
    if (!resident) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dem_end<ND, false>, BLK, 0);
        resident = std::max(1, sms * per_sm);
    }
    return std::max(1, std::min(resident, warp_blocks((int)std::min<int64_t>(particles, 1 << 22))));
}

/* list build: grid-stride over 32-particle slices, one wave of resident blocks */
template <int ND, bool COUNT>
int nlist_blocks(int64_t particles) {
    static int resident = 0;
    if (!resident) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_nlist<ND, COUNT>, NL_WARPS * 32, 0);
        resident = std::max(1, sms * per_sm);
    }
    const int64_t need = (particles + 32 * NL_WARPS - 1) / (32 * NL_WARPS);
    return (int)std::max<int64_t>(1, std::min<int64_t>(resident, need));
}

}  // namespace

void mixed_list_export(sphdem_ctx *c, int *cnt, const long long *offs, int *idx) {
    k_list_export<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n,
                                                              cnt, offs, idx);
}

void mixed_adj_pairs(sphdem_ctx *c, int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot) {
    const int g = grid_for(c->n, 128);
    if (c->cfg.nd == 3)
        k_adj_pairs<3><<<g, 128, 0, c->stream>>>(c->A, c->g, c->buf.skey, c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn,
                                                 c->n, nb, oc, cnt, cap, slot);
    else if (c->cfg.nd == 2)
        k_adj_pairs<2><<<g, 128, 0, c->stream>>>(c->A, c->g, c->buf.skey, c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn,
                                                 c->n, nb, oc, cnt, cap, slot);
    else
        k_adj_pairs<1><<<g, 128, 0, c->stream>>>(c->A, c->g, c->buf.skey, c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn,
                                                 c->n, nb, oc, cnt, cap, slot);
}

/* ---------------------------------------------------------------------- */
#define SPHDEM_ND_DISPATCH(nd, F) \
    do {                          \
        if ((nd) == 3) {          \
            F(3);                 \
        } else if ((nd) == 2) {   \
            F(2);                 \
        } else {                  \
            F(1);                 \
        }                         \
    } while (0)

namespace mixed {

void pack(sphdem_ctx *c, bool coupling) {
    coupling = coupling && c->cfg.liq_dem();
#define L_(ND)                                                                                                  \
    SPHDEM_LAUNCH(c, "pack32", k_pack<ND>, grid_for(c->n, 256), 256, 0, c->cfg, c->A, c->buf.skey, c->g,         \
                  c->mx_pos, c->mx_vel, c->mx_aux, c->mx_poslo, c->mx_tg, c->mx_rc4, (int)coupling, c->mx_ds,      \
                  c->mx_nb, c->n)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
    if (coupling) {
#define L_(ND)                                                                                                  \
    SPHDEM_LAUNCH(c, "couple_win", k_win<ND>, grid_for(3 * (int64_t)c->mx_win_cap, 256), 256, 0, c->cfg, c->g,   \
                  c->mx_win, c->mx_win_cap)
        SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
    }
}

void zero_shep(sphdem_ctx *c) {
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(c->mx_shep32, 0, c->n * sizeof(float), c->stream));
}

void pack_fpi(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "pack_fpi32", k_pack_fpi, grid_for(c->n, 256), 256, 0, c->A, c->mx_q0, c->mx_q1, c->mx_q2, c->n);
}

int band_records_per_particle() { return NL_QB; }

void nlist(sphdem_ctx *c) {
#define L_(ND)                                                                                                  \
    SPHDEM_LAUNCH(c, "nlist32", (k_nlist<ND, false>), (std::max(1, nlist_blocks<ND, false>(c->n) / c->grid_div)), NL_WARPS * 32, 0, c->cfg,  \
                  c->A, c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_tg, c->mx_nbr, c->mx_ncnt, c->mx_maxn,  \
                  c->cap, c->mx_bandq, c->mx_bandn)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
#define L_(ND)                                                                                                  \
    SPHDEM_LAUNCH(c, "band_fix", k_band_fix<ND>, grid_for(c->n, 256), 256, 0, c->cfg, c->A, c->g, c->buf.start,  \
                  c->buf.skey, c->mx_pos, c->mx_poslo, c->mx_bandq, c->mx_bandn, c->mx_nbr, (int64_t)c->mx_maxn)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
}

/* largest neighbour count at the current positions (sizes the lists); band
 * candidates count as neighbours, so this is an upper bound */
int nlist_max_count(sphdem_ctx *c) {
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(c->mx_ncnt, 0, c->n * sizeof(int), c->stream));
#define L_(ND)                                                                                                    \
    k_nlist<ND, true><<<nlist_blocks<ND, true>(c->n), NL_WARPS * 32, 0, c->stream>>>(                           \
        c->cfg, c->A, c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_tg, c->mx_nbr, c->mx_ncnt, 0, c->cap,     \
        nullptr, nullptr)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    std::vector<int> h(c->n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(h.data(), c->mx_ncnt, c->n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    int m = 0;
    for (int v : h) m = std::max(m, v);
    return m;
}

void omega_eos(sphdem_ctx *c, bool omega, bool eos) {
#define L_(ND)                                                                                                  \
    SPHDEM_LAUNCH(c, omega ? "omega_eos32" : "eos32", k_omega_eos<ND>, grid_for(c->n, c->blk_pair), c->blk_pair, 0, \
                  c->cfg, c->A, \
                  c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n,         \
                  (int)omega, (int)eos, c->mx_om)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
}

void force(sphdem_ctx *c) {
    const int phys = phys_class(c->cfg);
    const double *cgrows = corrected_gradient(c) ? c->cg : nullptr;
    /* neighbour records staged through shared memory (2D and 3D) */
    const bool tile = c->cfg.nd > 1 && c->force_tile;
    const size_t st_bytes = tile ? (size_t)3 * ST_CAP * sizeof(float4) : 0;
#define LP_(ND, P)                                                                                              \
    do {                                                                                                        \
        if (tile) {                                                                                             \
            SPHDEM_LAUNCH(c, "force32", (k_force<ND, P, true>), grid_for(c->n, c->blk_pair), c->blk_pair,      \
                          st_bytes, c->cfg, c->dcfg, c->A, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_om,     \
                          c->mx_tg, c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n, c->mx_nb, cgrows,        \
                          c->buf.start, c->buf.skey);                                                          \
        } else {                                                                                                \
            SPHDEM_LAUNCH(c, "force32", (k_force<ND, P, false>), grid_for(c->n, c->blk_pair), c->blk_pair, 0,  \
                          c->cfg, c->dcfg, c->A, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_om, c->mx_tg,     \
                          c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n, c->mx_nb, cgrows, c->buf.start,    \
                          c->buf.skey);                                                                        \
        }                                                                                                       \
    } while (0)
#define L_(ND)                                                                                                  \
    do {                                                                                                        \
        if (cgrows) {                                                                                           \
            LP_(ND, PHYS_CG);                                                                                   \
            break;                                                                                              \
        }                                                                                                       \
        if constexpr (ND > 1) {                                                                                 \
            if (phys == PHYS_MORRIS_VARH) {                                                                     \
                LP_(ND, PHYS_MORRIS_VARH);                                                                      \
                break;                                                                                          \
            }                                                                                                   \
            if (phys == PHYS_ARTIFICIAL) {                                                                      \
                LP_(ND, PHYS_ARTIFICIAL);                                                                       \
                break;                                                                                          \
            }                                                                                                   \
        }                                                                                                       \
        LP_(ND, PHYS_GENERIC);                                                                                  \
    } while (0)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
#undef LP_
}

/* Kernel attributes the step needs, set once per process outside any
 * stream capture: the dynamic shared memory of the staged force passes. */
void prepare(sphdem_ctx *) {
    static bool done = false;
    if (done) return;
    const int bytes = (int)(3 * ST_CAP * sizeof(float4));
#define A_(ND, P) \
    SPHDEM_CUDA_CHECK(cudaFuncSetAttribute(k_force<ND, P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))
    A_(2, PHYS_GENERIC);
    A_(2, PHYS_MORRIS_VARH);
    A_(2, PHYS_ARTIFICIAL);
    A_(2, PHYS_CG);
    A_(3, PHYS_GENERIC);
    A_(3, PHYS_MORRIS_VARH);
    A_(3, PHYS_ARTIFICIAL);
    A_(3, PHYS_CG);
#undef A_
    const int bytes2 = (int)(2 * ST_CAP * sizeof(float4));
#define D_(ND, CGF, VH) \
    SPHDEM_CUDA_CHECK(cudaFuncSetAttribute(k_dddt<ND, CGF, VH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes2))
    D_(2, true, -1);
    D_(2, false, 1);
    D_(2, false, 0);
    D_(3, true, -1);
    D_(3, false, 1);
    D_(3, false, 0);
#undef D_
    done = true;
}

void dddt(sphdem_ctx *c) {
    const double *cgrows = corrected_gradient(c) ? c->cg : nullptr;
    const bool vh = c->cfg.var_h();
    const bool tile = c->cfg.nd > 1 && c->force_tile;
    const size_t st_bytes = (size_t)2 * ST_CAP * sizeof(float4);
#define LD_(ND, CGF, VH)                                                                                        \
    do {                                                                                                        \
        if (tile)                                                                                               \
            SPHDEM_LAUNCH(c, "dddt32", (k_dddt<ND, CGF, VH, true>), grid_for(c->n, c->blk_pair), c->blk_pair,  \
                          st_bytes, c->cfg, c->A, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_om, c->mx_tg,    \
                          c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n, cgrows, c->buf.start, c->buf.skey); \
        else                                                                                                    \
            SPHDEM_LAUNCH(c, "dddt32", (k_dddt<ND, CGF, VH, false>), grid_for(c->n, c->blk_pair), c->blk_pair, \
                          0, c->cfg, c->A, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_om, c->mx_tg,           \
                          c->mx_nbr, c->mx_ncnt, (int64_t)c->mx_maxn, c->n, cgrows, c->buf.start, c->buf.skey); \
    } while (0)
#define L_(ND)                       \
    do {                             \
        if (cgrows)                  \
            LD_(ND, true, -1);       \
        else if (vh)                 \
            LD_(ND, false, 1);       \
        else                         \
            LD_(ND, false, 0);       \
    } while (0)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
#undef LD_
}

/* the porosity (MODE 0) or DEM -> SPH drag (MODE 1) pass; while the
 * adjoint's replay graph is captured, the form that also writes the
 * coupling tap table */
template <int MODE>
void couple(sphdem_ctx *c, const char *name) {
    const TapTable tt = c->tap ? c->tap->cpl : TapTable{};
    const int *ts = c->tap ? c->tap->slot : nullptr;
#define L_(ND)                                                                                                  \
    do {                                                                                                        \
        const int nb_ = std::max(1, resident_blocks<ND, MODE>(c->n) / c->grid_div);                             \
        if (c->tap)                                                                                             \
            SPHDEM_LAUNCH(c, name, (k_couple<ND, MODE, true>), nb_, CP_WARPS * 32, 0, c->cfg, c->dcfg, c->A,      \
                          c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_dp, c->mx_tg,   \
                          c->mx_rc4, c->mx_win, c->mx_win_cap, c->mx_shep32, tt, ts, c->n);                       \
        else                                                                                                    \
            SPHDEM_LAUNCH(c, name, (k_couple<ND, MODE, false>), nb_, CP_WARPS * 32, 0, c->cfg, c->dcfg, c->A,     \
                          c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_vel, c->mx_aux, c->mx_dp, c->mx_tg,   \
                          c->mx_rc4, c->mx_win, c->mx_win_cap, c->mx_shep32, tt, ts, c->n);                       \
    } while (0)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
}

void porosity(sphdem_ctx *c) { couple<0>(c, "porosity32"); }

void dem_drag(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "pack_dem_drag32", k_pack_dem_drag, grid_for(c->n, 256), 256, 0, c->A, c->mx_shep32, c->mx_vel,
                  c->mx_dp, c->n);
    couple<1>(c, "dem_drag32");
}

void dem_end(sphdem_ctx *c) {
    pack_fpi(c);
    /* one warp per DEM particle, grid-stride over the DEM range: one wave of
     * resident blocks (a grid sized by the particle count would launch
     * mostly empty warps) */
    const TapTable tf = c->tap ? c->tap->fpi : TapTable{}, tct = c->tap ? c->tap->ct : TapTable{};
    const int *ts = c->tap ? c->tap->slot : nullptr;
#define L_(ND)                                                                                                  \
    do {                                                                                                        \
        if (c->tap)                                                                                             \
            SPHDEM_LAUNCH(c, "dem_end32", (k_dem_end<ND, true>), dem_end_blocks<ND>(c->n), BLK, 0, c->cfg,        \
                          c->dcfg, c->A, c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_vel, c->mx_aux,        \
                          c->mx_q0, c->mx_q1, c->mx_q2, c->mx_tg, c->mx_ds, tf, tct, ts, c->n);                   \
        else                                                                                                    \
            SPHDEM_LAUNCH(c, "dem_end32", (k_dem_end<ND, false>), dem_end_blocks<ND>(c->n), BLK, 0, c->cfg,       \
                          c->dcfg, c->A, c->buf.start, c->buf.skey, c->g, c->mx_pos, c->mx_vel, c->mx_aux,        \
                          c->mx_q0, c->mx_q1, c->mx_q2, c->mx_tg, c->mx_ds, tf, tct, ts, c->n);                   \
    } while (0)
    SPHDEM_ND_DISPATCH(c->cfg.nd, L_);
#undef L_
}

}  // namespace mixed
}  // namespace sphdem
