/*
 * Mixed-precision pair passes (SPHDEM_PREC_MIXED).
 *
 * Positions stay FP64 in the state; for the pair math every particle is
 * packed, once per rebuild, as an FP32 offset from the FP64 origin of its own
 * bucket plus FP32 h / velocity / mass / density / pdr2.  The displacement of
 * a pair in buckets ca and cb = ca + o is then (off_a - off_b) - o*bucket, all
 * FP32 and well conditioned (|off| < one bucket).
 *
 *   k_nlist     after each rebuild, the exact neighbour list of every
 *               sph/sphBoundary particle: one warp per SPH bucket walks the
 *               3^d stencil with warp-uniform loads, FP32 distance test, and
 *               the FP64 predicate of the reference (particle.h:236-238) inside
 *               a 4e-6 relative band around the cut-off; periodic images only
 *               where the reference holds a ghost.  Stored column-major
 *               (entry j of all particles contiguous) as b | stencil code << 26.
 *   k_omega32   calcOmega (+ the FP64 EOS, whose (rho/rho0)^7-1 cancels too
 *               much for FP32) over the list
 *   k_force32   calcForce + dt conditions over the list
 *   k_dddt32    calcDddtDudt over the list
 *   k_porosity32 / k_dem_drag32 / k_dem_end32: the coupling and DEM passes,
 *               bucket stencils in FP32 with the same exact band tests.
 *
 * Sums are Kahan-compensated in FP32 and added to the FP64 state once per
 * particle.  Roofline: FP32-pipe-bound for the list passes on 3D workloads
 * (~100 FP32 ops per listed pair against 48 B of packed input per particle).
 */
#include <algorithm>
#include <cfloat>
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
};

struct Grid32 {
    int dims[3];
    float cell[3];      /* bucket size per axis, FP32 */
    int n_sph_cells;
};

__device__ __forceinline__ Grid32 sph_grid32(const DevCfg &c, const DevGlobals *g) {
    Grid32 G;
    for (int d = 0; d < 3; d++) {
        G.dims[d] = g->sdims[d];
        G.cell[d] = (float)(c.periodic[d] ? g->scell[d] : g->sr2);
    }
    G.n_sph_cells = g->n_sph_cells;
    return G;
}

__device__ __forceinline__ Grid32 dem_grid32(const DevCfg &c, const DevGlobals *g) {
    Grid32 G;
    for (int d = 0; d < 3; d++) {
        G.dims[d] = c.ddims[d];
        G.cell[d] = (float)c.dcell[d];
    }
    G.n_sph_cells = g->n_sph_cells;
    return G;
}

/* FP64 origin of SPH bucket `cell` on axis d */
__device__ __forceinline__ double sph_origin(const DevCfg &c, const DevGlobals *g, int d, int cell) {
    return c.periodic[d] ? c.dmin[d] + cell * g->scell[d] : c.dmin[d] + (cell - 3) * g->sr2;
}
__device__ __forceinline__ double dem_origin(const DevCfg &c, int d, int cell) {
    return c.dorig[d] + cell * c.dcell[d];
}

__device__ __forceinline__ CellCoord sph_cell_of(const DevCfg &c, const DevGlobals *g, const double *r) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    for (int d = 0; d < c.nd; d++) {
        int k = c.periodic[d] ? (int)floor((r[d] - c.dmin[d]) * g->rscell[d])
                              : trunc_index(r[d], c.dmin[d], g->sr2, g->rsr2_f, 3.0);
        k = k < 0 ? 0 : (k >= g->sdims[d] ? g->sdims[d] - 1 : k);
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

__device__ __forceinline__ int ocode(int ox, int oy, int oz) { return (ox + 1) * 9 + (oy + 1) * 3 + (oz + 1); }
__device__ __forceinline__ void odecode(int code, int *o) {
    o[0] = code / 9 - 1;
    o[1] = (code / 3) % 3 - 1;
    o[2] = code % 3 - 1;
}

/* exact FP64 predicate of the reference for a pair near the cut-off */
__device__ __noinline__ bool exact_pair(const DevCfg &c, const DevState &s, int a, int b, const int *sh, double rad2_lim,
                                        bool strict) {
    double dx[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++)
        dx[d] = dsub(s.row(FD_R + d)[a], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
    const double r2 = exact_len2(dx, c.nd);
    if (rad2_lim > 0) return strict ? r2 < rad2_lim : r2 <= rad2_lim;
    const double ha = s.row(FD_H)[a], hb = s.row(FD_H)[b];
    const double t = 2.0 * (ha > hb ? ha : hb);
    return r2 <= dmul(t, t);
}

/* ---------------------------------------------------------------------- */
/* packing: P0 = (offset from own bucket origin, h), P1 = (vhat, mass),
 * P2 = (dens, pdr2, porosity, 1/h), tg = type | gcode << 8 */
__global__ void k_pack(DevCfg c, DevState s, const int *skey, const DevGlobals *g, float4 *P0, float4 *P1,
                       float4 *P2, int *tg, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    tg[i] = (t & 0xff) | (s.irow(FI_GCODE)[i] << 8);
    if (t == T_DEAD) return;
    const int key = skey[i];
    float off[3] = {0.f, 0.f, 0.f};
    if (c.liq_dem() && t == T_DEM) {
        const CellCoord cc = decode_cell(key - g->n_sph_cells, c.ddims, c.nd);
        for (int d = 0; d < c.nd; d++) off[d] = (float)(s.row(FD_R + d)[i] - dem_origin(c, d, cc.c[d]));
    } else {
        int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
        const CellCoord cc = decode_cell(key, dims, c.nd);
        for (int d = 0; d < c.nd; d++) off[d] = (float)(s.row(FD_R + d)[i] - sph_origin(c, g, d, cc.c[d]));
    }
    const double h = s.row(FD_H)[i];
    P0[i] = make_float4(off[0], off[1], off[2], (float)h);
    P1[i] = make_float4((float)s.row(FD_VHAT)[i], c.nd > 1 ? (float)s.row(FD_VHAT + 1)[i] : 0.f,
                        c.nd > 2 ? (float)s.row(FD_VHAT + 2)[i] : 0.f, (float)s.row(FD_MASS)[i]);
    P2[i] = make_float4((float)s.row(FD_DENS)[i], (float)s.row(FD_PDR2)[i], (float)s.row(FD_POR)[i],
                        (float)s.row(FD_IH)[i]);
}

/* ---------------------------------------------------------------------- */
__global__ void k_nlist(DevCfg c, DevState s, const int *start, const DevGlobals *g, const float4 *P0, const int *tg,
                        int *nbr, int *ncnt, int maxn, int64_t ld, int count_only) {
    const int lane = threadIdx.x & 31;
    const int warps = (blockDim.x >> 5) * gridDim.x;
    const Grid32 G = sph_grid32(c, g);
    for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < G.n_sph_cells; cell += warps) {
        const int s0 = start[cell], s1 = start[cell + 1];
        if (s0 == s1) continue;
        const CellCoord cc = decode_cell(cell, G.dims, c.nd);
        for (int base = s0; base < s1; base += 32) {
            const int a = base + lane;
            const bool act = a < s1 && is_sph_or_sphb(tg[a] & 0xff);
            float4 pa = make_float4(0, 0, 0, 0);
            if (act) pa = P0[a];
            int cnt = 0;
            for (int ox = -1; ox <= 1; ox++)
                for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
                    for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                        int sh[3];
                        const int lin = neighbour_cell(cc, ox, oy, oz, G.dims, c.periodic, c.nd, sh);
                        if (lin < 0) continue;
                        const int b0 = start[lin], b1 = start[lin + 1];
                        const float dx0 = -ox * G.cell[0], dy0 = -oy * G.cell[1], dz0 = -oz * G.cell[2];
                        const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
                        const int code = ocode(ox, oy, oz) << B_BITS;
                        for (int b = b0; b < b1; b++) {
                            const float4 pb = P0[b];
                            if (!act) continue;
                            if (b == a && !shifted) continue;
                            const float dx = pa.x - pb.x + dx0, dy = pa.y - pb.y + dy0, dz = pa.z - pb.z + dz0;
                            const float r2 = dx * dx + dy * dy + dz * dz;
                            const float t = 2.f * fmaxf(pa.w, pb.w);
                            const float T = t * t;
                            bool in;
                            if (r2 < T * (1.f - 4e-6f)) in = true;
                            else if (r2 > T * (1.f + 4e-6f)) in = false;
                            else in = exact_pair(c, s, a, b, sh, 0.0, false);
                            if (in && shifted) in = image_exists(tg[b] >> 8, sh, c.nd);
                            if (in) {
                                if (cnt < maxn) nbr[(int64_t)cnt * ld + a] = b | code;
                                cnt++;
                            }
                        }
                    }
            if (act) {
                /* stored counts never exceed the list depth; an overflow is an error */
                ncnt[a] = count_only ? cnt : min(cnt, maxn);
                if (cnt > maxn && !count_only) set_err(const_cast<DevGlobals *>(g), SPHDEM_ERR_CAPACITY, cnt);
            }
        }
    }
}

__device__ __forceinline__ void nb_delta(int e, const Grid32 &G, float4 pa, float4 pb, float *d) {
    int o[3];
    odecode(e >> B_BITS, o);
    d[0] = pa.x - pb.x - o[0] * G.cell[0];
    d[1] = pa.y - pb.y - o[1] * G.cell[1];
    d[2] = pa.z - pb.z - o[2] * G.cell[2];
}

/* ---------------------------------------------------------------------- */
/* calcOmega (sph.h:438-451) over the list, then the FP64 EOS */
__global__ void k_omega_eos32(DevCfg c, DevState s, const DevGlobals *g, const float4 *P0, const float4 *P1,
                              float4 *P2, const int *tg, const int *nbr, const int *ncnt, int64_t ld, int64_t n,
                              int do_omega, int do_eos, float *om32) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    const Grid32 G = sph_grid32(c, g);
    const float wcon = (float)c.wcon;
    if (do_omega) {
        const float4 pa = P0[a];
        const float iha = 1.f / pa.w;
        float ihna = iha;
        for (int d = 1; d < c.nd; d++) ihna *= iha;
        const float pd_coef = c.nd * ihna * iha;
        const double ha = s.row(FD_H)[a];
        Kahan om;
        om.init(-P1[a].w * pd_coef * wK32(0.f, wcon));
        const int cnt = ncnt[a];
        for (int j = 0; j < cnt; j++) {
            const int e = nbr[(int64_t)j * ld + a];
            const int b = e & B_MASK;
            if (!is_sph_or_sphb(tg[b] & 0xff)) continue;
            const float4 pb = P0[b];
            float d[3];
            nb_delta(e, G, pa, pb, d);
            const float r = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const float q = r * iha;
            const float pdkh = -q * wdK32(q, wcon) * iha;
            om.add(P1[b].w * (ihna * pdkh - pd_coef * wK32(q, wcon)));
        }
        const double omega = 1 + ha * (double)om.s / (s.row(FD_DENS)[a] * c.nd);
        s.row(FD_OMEGA)[a] = omega;
        om32[a] = (float)omega;
    }
    if (do_eos) {
        const double densa = s.row(FD_DENS)[a];
        const double x = c.liq_dem() ? densa / (c.refd * s.row(FD_POR)[a]) : densa / c.refd;
        double xg;
        if (!c.liq_dem() || c.gamma == 7.0) {
            const double x2 = x * x;
            xg = x2 * x2 * x2 * x;
        } else {
            xg = pow(x, c.gamma);
        }
        const double press = c.prb * (xg - 1.0);
        const double pdr2 = press / (densa * densa);
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
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) smin[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? smin[lane] : FLT_MAX;
        for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v < FLT_MAX) atomic_min_pos(target, (double)v);
    }
}

/* calcForce + calcViscForce + calcPressForce + boundary force (FP32) */
__global__ void __launch_bounds__(BLK) k_force32(DevCfg c, DevState s, DevGlobals *g, const float4 *P0,
                                                 const float4 *P1, const float4 *P2, const float *om32,
                                                 const int *tg, const int *nbr, const int *ncnt, int64_t ld,
                                                 int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float ndt = FLT_MAX;
    const int ta = a < n ? (tg[a] & 0xff) : -1;
    if (is_sph_or_sphb(ta)) {
        const Grid32 G = sph_grid32(c, g);
        const float wcon = (float)c.wcon;
        const float4 pa = P0[a], va = P1[a], xa = P2[a];
        const float ha = pa.w, iha = xa.w;
        float ihn2a = iha * iha;
        for (int d = 0; d < c.nd; d++) ihn2a *= iha;
        const float densa = xa.x, pdr2a = xa.y, ma = va.w;
        const float roma = c.var_h() ? 1.f / om32[a] : 1.f;
        const bool sph = ta == T_SPH;
        const bool anti = !(c.flags & SPHDEM_F_NO_ANTICLUMPING);
        const float visc_nu = (float)c.viscosity, c0 = (float)c.spsound;
        const float liq_visc = (float)(2.0 * c.viscosity * c.dens);
        const float alpha_mon = (float)c.alpha_mon, alpha_art = (float)c.alpha_art;
        const float vdc = c.visc == SPHDEM_VISC_MONAGHAN ? 0.06f : 0.125f;
        const float k_anti_inv = c.k_anti != 0 ? (float)(1.0 / c.k_anti) : 0.f;
        Kahan fp[3], fv[3], fb[3], fa[3];
        for (int d = 0; d < 3; d++) {
            fp[d].init(0.f);
            fv[d].init(0.f);
            fb[d].init(0.f);
            fa[d].init(0.f);
        }
        const int cnt = ncnt[a];
        for (int j = 0; j < cnt; j++) {
            const int e = nbr[(int64_t)j * ld + a];
            const int b = e & B_MASK;
            const int tb = tg[b] & 0xff;
            const float4 pb = P0[b], vb = P1[b], xb = P2[b];
            float d[3];
            nb_delta(e, G, pa, pb, d);
            const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
            const float r = r2 * rinv;
            const float hb = pb.w, ihb = xb.w;
            float ihn2b = ihb * ihb;
            for (int k = 0; k < c.nd; k++) ihn2b *= ihb;
            const float qa = r * iha, qb = r * ihb;
            /* dr*F(q,h) with F = ihn2*dK/dq/q and 1/q = h/r */
            const float Fa = qa != 0.f ? ihn2a * wdK32(qa, wcon) * (ha * rinv) : 0.f;
            const float Fb = qb != 0.f ? ihn2b * wdK32(qb, wcon) * (hb * rinv) : 0.f;
            float gA[3], gB[3], gm[3];
            if (c.var_h()) {
                for (int k = 0; k < 3; k++) {
                    gA[k] = d[k] * Fa * roma;
                    gB[k] = d[k] * Fb * roma;
                    gm[k] = 0.5f * (gA[k] + gB[k]);
                }
            } else {
                for (int k = 0; k < 3; k++) {
                    gA[k] = gB[k] = gm[k] = 0.5f * (d[k] * Fa + d[k] * Fb);
                }
            }
            const float densb = xb.x, mb = vb.w;
            const float hav = 0.5f * (ha + hb);
            if (sph && tb != T_DEM && tb != T_DEMB) {
                const float dv0 = va.x - vb.x, dv1 = va.y - vb.y, dv2 = va.z - vb.z;
                const float vdr = d[0] * dv0 + d[1] * dv1 + d[2] * dv2;
                float vsig = 0.f;
                if (c.visc == SPHDEM_VISC_MORRIS) {
                    const float visc = c.liq_dem() ? liq_visc / (densa * densb)
                                                   : visc_nu * (densa + densb) / (densa * densb);
                    vsig = 2.f * c0;
                    const float dg = d[0] * gm[0] + d[1] * gm[1] + d[2] * gm[2];
                    const float sc = mb * visc * dg / (r * r + 0.01f * hav * hav);
                    fv[0].add(dv0 * sc);
                    fv[1].add(dv1 * sc);
                    fv[2].add(dv2 * sc);
                } else if (c.visc == SPHDEM_VISC_MONAGHAN) {
                    const float viss = vdr * rinv;
                    if (!c.liq_dem()) vsig = 2.f * c0 + 2.f * fabsf(viss);
                    const float sc = mb * (viss * vsig * alpha_mon / (densa + densb));
                    for (int k = 0; k < 3; k++) fv[k].add(sc * gm[k]);
                } else if (c.visc == SPHDEM_VISC_ARTIFICIAL) {
                    if (vdr < 0.f) {
                        const float viss = vdr * rinv;
                        const float avsig = 2.f * c0 - 4.f * viss;
                        const float sc = mb * (viss * avsig * alpha_art / (densa + densb));
                        for (int k = 0; k < 3; k++) fa[k].add(sc * gm[k]);
                        vsig = fmaxf(vsig, avsig);
                    }
                }
                ndt = fminf(ndt, 0.6f * hav / vsig);
                ndt = fminf(ndt, vdc * hav * hav / visc_nu);
            }
            float kdw4 = 0.f;
            if (anti) {
                const float kdw = wK32(r / hav, wcon) * k_anti_inv;
                kdw4 = (kdw * kdw) * (kdw * kdw);
            }
            if (is_boundary(tb)) {
                /* calcNormal + calcBoundaryForces (sph.h:736-918) */
                float n1[3] = {0, 0, 0}, n2[3] = {0, 0, 0}, nt[3] = {0, 0, 0}, np[3];
                for (int k = 0; k < c.nd; k++) {
                    n1[k] = (float)s.row(FD_N1 + k)[b];
                    n2[k] = (float)s.row(FD_N2 + k)[b];
                    nt[k] = c.nd == 3 ? (float)s.row(FD_N3 + k)[b] : 0.f;
                }
                if (n2[0] == 0.f && n2[1] == 0.f && n2[2] == 0.f) {
                    for (int k = 0; k < 3; k++) np[k] = n1[k];
                } else {
                    const float rd1 = d[0] * n1[0] + d[1] * n1[1] + d[2] * n1[2];
                    const float rd2 = d[0] * n2[0] + d[1] * n2[1] + d[2] * n2[2];
                    const float rnt = r * r * (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) - rd1 * rd2;
                    if (rnt <= 0.f) {
                        for (int k = 0; k < 3; k++) np[k] = d[k] * rinv;
                    } else {
                        const int con = s.irow(FI_CONCAVE)[b] ? 1 : -1;
                        for (int k = 0; k < 3; k++) np[k] = con * (rd1 - rd2) > 0.f ? n1[k] : n2[k];
                    }
                }
                const float dv0 = va.x - vb.x, dv1 = va.y - vb.y, dv2 = va.z - vb.z;
                const float rperp = np[0] * d[0] + np[1] * d[1] + np[2] * d[2];
                const float rt0 = d[0] - rperp * np[0], rt1 = d[1] - rperp * np[1], rt2 = d[2] - rperp * np[2];
                const float rdelp = (float)(1.0 / (c.bfac * c.psep));
                float pt0, pt1;
                if (c.nd == 3) {
                    pt0 = fabsf(rt0 * nt[0] + rt1 * nt[1] + rt2 * nt[2]);
                    const float c0x = rt1 * nt[2] - rt2 * nt[1], c1x = rt2 * nt[0] - rt0 * nt[2],
                                c2x = rt0 * nt[1] - rt1 * nt[0];
                    pt1 = sqrtf(c0x * c0x + c1x * c1x + c2x * c2x);
                } else {
                    pt0 = sqrtf(rt0 * rt0 + rt1 * rt1);
                    pt1 = 0.f;
                }
                const float pd0 = pt0 * rdelp, pd1 = pt1 * rdelp;
                if (pd0 <= 1.f && pd1 <= 1.f) {
                    const float pif = (float)c.pi;
                    const float pesky = 0.25f * (1.f + cosf(pif * pd0)) * (1.f + cosf(pif * pd1));
                    const float q = fabsf(rperp) * (float)(1.0 / c.psep);
                    if (q < 2.f) {
                        const int beta = (d[0] * dv0 + d[1] * dv1 + d[2] * dv2) < 0.f ? 1 : 0;
                        const float bigA = 0.01f * c0 * c0 - beta * c0 * (dv0 * np[0] + dv1 * np[1] + dv2 * np[2]);
                        const float bfact = 1.f / fabsf(rperp);
                        const float QIN = 2.f / 3.f;
                        float bforce = 0.f;
                        if (q <= QIN) bforce = bfact * QIN;
                        else if (q <= 1.f) bforce = bfact * (2.f * q - 1.5f * q * q);
                        else bforce = bfact * 0.5f * (2.f - q) * (2.f - q);
                        const float amassrat = 2.f * ma / (ma + mb);
                        const float sgn = rperp < 0.f ? -1.f : 1.f;
                        const float sc = sgn * amassrat * bigA * bforce * pesky;
                        for (int k = 0; k < 3; k++) fb[k].add(sc * np[k]);
                    }
                }
            } else if (tb == T_SPH || tb == T_SPHB) {
                const float pdr2b = xb.y;
                const float antic = 0.01f * fabsf(pdr2a + pdr2b) * kdw4;
                for (int k = 0; k < c.nd; k++) fp[k].add(-mb * ((pdr2a * gA[k] + pdr2b * gB[k]) + antic));
            }
        }
        double fsum2 = 0.0;
        for (int k = 0; k < c.nd; k++) {
            double *f = s.row(FD_F + k);
            const double fpk = (double)fp[k].s - (double)fp[k].c;
            const double fvk = (double)fv[k].s - (double)fv[k].c;
            const double fbk = (double)fb[k].s - (double)fb[k].c;
            const double fak = (double)fa[k].s - (double)fa[k].c;
            s.row(FD_FP + k)[a] += fpk;
            s.row(FD_FV + k)[a] += fvk;
            s.row(FD_FB + k)[a] += fbk;
            const double fk = f[a] + fak + fvk + fbk + fpk;
            f[a] = fk;
            fsum2 += fk * fk;
        }
        ndt = fminf(ndt, (float)(0.25 * sqrt((double)ha / sqrt(fsum2))));
    }
    block_min_atomic(ndt, &g->new_dt_bits);
}

/* calcDddtDudt (sphIncompress.h:783-851) over the list */
__global__ void __launch_bounds__(BLK) k_dddt32(DevCfg c, DevState s, const DevGlobals *g, const float4 *P0,
                                                const float4 *P1, const float4 *P2, const float *om32,
                                                const int *tg, const int *nbr, const int *ncnt, int64_t ld,
                                                int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    const Grid32 G = sph_grid32(c, g);
    const float wcon = (float)c.wcon;
    const float4 pa = P0[a], va = P1[a], xa = P2[a];
    const float ha = pa.w, iha = xa.w;
    float ihn2a = iha * iha;
    for (int d = 0; d < c.nd; d++) ihn2a *= iha;
    const float roma = c.var_h() ? 1.f / om32[a] : 1.f;
    Kahan acc;
    acc.init(0.f);
    const int cnt = ncnt[a];
    for (int j = 0; j < cnt; j++) {
        const int e = nbr[(int64_t)j * ld + a];
        const int b = e & B_MASK;
        const int tb = tg[b] & 0xff;
        if (is_boundary(tb) || tb == T_DEM) continue;
        const float4 pb = P0[b], vb = P1[b];
        float d[3];
        nb_delta(e, G, pa, pb, d);
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
        const float r = r2 * rinv;
        const float qa = r * iha;
        const float Fa = qa != 0.f ? ihn2a * wdK32(qa, wcon) * (ha * rinv) : 0.f;
        float F;
        if (c.var_h()) {
            F = Fa * roma;
        } else {
            const float ihb = P2[b].w, hb = pb.w;
            float ihn2b = ihb * ihb;
            for (int k = 0; k < c.nd; k++) ihn2b *= ihb;
            const float qb = r * ihb;
            const float Fb = qb != 0.f ? ihn2b * wdK32(qb, wcon) * (hb * rinv) : 0.f;
            F = 0.5f * (Fa + Fb);
        }
        const float vdr = (va.x - vb.x) * d[0] + (va.y - vb.y) * d[1] + (va.z - vb.z) * d[2];
        acc.add(vb.w * vdr * F);
    }
    s.row(FD_DDDT)[a] += (double)acc.s - (double)acc.c;
}

/* ---------------------------------------------------------------------- */
/* SPH -> DEM coupling over the DEM grid (calcNeighboursCoupling rule) */
template <class Body>
__device__ __forceinline__ void couple32(const DevCfg &c, const DevState &s, const int *start, const DevGlobals *g,
                                         const float4 *P0, const int *tg, int a, Body &&body) {
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    int cs[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) cs[d] = ref_dem_cell(ra[d], c, d);
    const CellCoord cc = dem_cell_of(c, ra);
    float oa[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) oa[d] = (float)(ra[d] - dem_origin(c, d, cc.c[d]));
    const Grid32 G = dem_grid32(c, g);
    const float rc2 = (float)c.rc2;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
            for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cc, ox, oy, oz, G.dims, c.periodic, c.nd, sh);
                if (lin < 0) continue;
                const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
                const int b0 = start[G.n_sph_cells + lin], b1 = start[G.n_sph_cells + lin + 1];
                for (int b = b0; b < b1; b++) {
                    if ((tg[b] & 0xff) != T_DEM) continue;
                    const float4 pb = P0[b];
                    float d[3];
                    d[0] = oa[0] - pb.x - ox * G.cell[0];
                    d[1] = oa[1] - pb.y - oy * G.cell[1];
                    d[2] = oa[2] - pb.z - oz * G.cell[2];
                    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    if (r2 > rc2 * (1.f + 4e-6f)) continue;
                    if (r2 >= rc2 * (1.f - 4e-6f) && !exact_pair(c, s, a, b, sh, c.rc2, true)) continue;
                    int cd[3] = {0, 0, 0};
                    for (int k = 0; k < c.nd; k++)
                        cd[k] = shifted ? ref_dem_cell(image_pos(s.row(FD_R + k)[b], sh[k], c.rmin[k], c.rmax[k]), c, k)
                                        : s.irow(FI_RDC0 + k)[b];
                    if (!coupling_rule(cs, cd, c)) continue;
                    if (shifted && !image_exists(tg[b] >> 8, sh, c.nd)) continue;
                    body(b, d, r2);
                }
            }
}

__global__ void k_porosity32(DevCfg c, DevState s, const int *start, const DevGlobals *g, const float4 *P0,
                             const float4 *P1, const int *tg, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(tg[a] & 0xff)) return;
    const float4 va = P1[a];
    const float dvol = (float)(s.row(FD_MASS)[a] / s.row(FD_DENS)[a]);
    const float two_over_rc = (float)c.two_over_rc, c_ihn = (float)c.c_ihn, c_ihn2 = (float)c.c_ihn2;
    const float wcon = (float)c.wcon, por_incr = (float)c.por_incr, dem_vol = (float)c.dem_vol;
    Kahan por, dpd, gp[3];
    por.init(0.f);
    dpd.init(0.f);
    for (int k = 0; k < 3; k++) gp[k].init(0.f);
    couple32(c, s, start, g, P0, tg, (int)a, [&](int b, const float *d, float r2) {
        const float r = sqrtf(r2);
        const float q = r * two_over_rc;
        const float Wa = c_ihn * wK32(q, wcon);
        por.add(por_incr * Wa);
        if (r != 0.f) {
            const float4 vb = P1[b];
            const float Fq = c_ihn2 * wdK32(q, wcon) / q;
            const float vd = (va.x - vb.x) * d[0] + (va.y - vb.y) * d[1] + (va.z - vb.z) * d[2];
            dpd.add(-dem_vol * vd * Fq);
            for (int k = 0; k < 3; k++) gp[k].add(dem_vol * d[k] * Fq);
        }
        atomicAdd(&s.row(FD_SHEP)[b], (double)(dvol * Wa));
    });
    s.row(FD_POR)[a] = (double)por.s - (double)por.c;
    s.row(FD_DPORDT)[a] = (double)dpd.s - (double)dpd.c;
    for (int k = 0; k < 3; k++) s.row(FD_GPOR + k)[a] = (double)gp[k].s - (double)gp[k].c;
}

__global__ void k_dem_drag32(DevCfg c, DevState s, const int *start, const DevGlobals *g, const float4 *P0,
                             const int *tg, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int t = tg[a] & 0xff;
    if (is_boundary(t)) {
        s.row(FD_POR)[a] = 1.0;
        return;
    }
    if (!is_sph_or_sphb(t)) return;
    const double densa = s.row(FD_DENS)[a];
    const float rdens = (float)(c.nd == 2 ? (1.0 / (2.0 * c.dem_radius)) / densa : 1.0 / densa);
    const float two_over_rc = (float)c.two_over_rc, c_ihn = (float)c.c_ihn, wcon = (float)c.wcon;
    Kahan fd[3];
    for (int k = 0; k < 3; k++) fd[k].init(0.f);
    couple32(c, s, start, g, P0, tg, (int)a, [&](int b, const float *d, float r2) {
        const float w = c_ihn * wK32(sqrtf(r2) * two_over_rc, wcon);
        const float sc = (float)(s.row(FD_MASS)[b] / s.row(FD_SHEP)[b]) * rdens * w;
        for (int k = 0; k < c.nd; k++) fd[k].add(-sc * (float)s.row(FD_FDRAG + k)[b]);
    });
    for (int k = 0; k < c.nd; k++) {
        const double v = (double)fd[k].s - (double)fd[k].c;
        s.row(FD_FDRAG + k)[a] = v;
        s.row(FD_F + k)[a] += v;
    }
    double por = 1.0 - s.row(FD_POR)[a];
    if (por < 0.37) {
        por = 0.37;
        s.row(FD_DPORDT)[a] = 0.0;
        for (int d = 0; d < 3; d++) s.row(FD_GPOR + d)[a] = 0.0;
    }
    s.row(FD_POR)[a] = por;
}

/* calcFPI + calcParticleDrag + calcDEMContacts for DEM particles (FP32 sums) */
__global__ void k_dem_end32(DevCfg c, DevState s, const int *start, const DevGlobals *g, const float4 *P0,
                            const float4 *P1, const float4 *P2, const int *tg, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if ((tg[a] & 0xff) != T_DEM) return;
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const float4 va = P1[a];
    const float ha = P0[a].w;
    const float wcon = (float)c.wcon;
    /* FPI over the SPH grid */
    const CellCoord cs = sph_cell_of(c, g, ra);
    float oa[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) oa[d] = (float)(ra[d] - sph_origin(c, g, d, cs.c[d]));
    const Grid32 GS = sph_grid32(c, g);
    Kahan sum, fdens, por, ff[3], fpfb[3], fv[3], fdr[3], fvel[3];
    sum.init(0.f);
    fdens.init(0.f);
    por.init(0.f);
    for (int k = 0; k < 3; k++) {
        ff[k].init(0.f);
        fpfb[k].init(0.f);
        fv[k].init(0.f);
        fdr[k].init(0.f);
        fvel[k].init(0.f);
    }
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
            for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cs, ox, oy, oz, GS.dims, c.periodic, c.nd, sh);
                if (lin < 0) continue;
                const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
                for (int b = start[lin]; b < start[lin + 1]; b++) {
                    const float4 pb = P0[b];
                    const float dx = oa[0] - pb.x - ox * GS.cell[0], dy = oa[1] - pb.y - oy * GS.cell[1],
                                dz = oa[2] - pb.z - oz * GS.cell[2];
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    const float t = 2.f * fmaxf(ha, pb.w);
                    const float T = t * t;
                    if (r2 > T * (1.f + 4e-6f)) continue;
                    if (r2 >= T * (1.f - 4e-6f) && !exact_pair(c, s, (int)a, b, sh, 0.0, false)) continue;
                    if (shifted && !image_exists(tg[b] >> 8, sh, c.nd)) continue;
                    if ((tg[b] & 0xff) == T_BOUNDARY) continue;
                    const float4 vb = P1[b], xb = P2[b];
                    const float mb = vb.w;
                    const float dvol = mb / xb.x;
                    const float q = sqrtf(r2) * xb.w;
                    float ihnb = xb.w;
                    for (int k = 1; k < c.nd; k++) ihnb *= xb.w;
                    const float Wab = ihnb * wK32(q, wcon);
                    const float dvW = dvol * Wab, mW = mb * Wab;
                    for (int k = 0; k < c.nd; k++) {
                        const float fvb = (float)s.row(FD_FV + k)[b];
                        fpfb[k].add(mW * (float)(s.row(FD_FP + k)[b] + s.row(FD_FB + k)[b]));
                        fv[k].add(mW * fvb);
                        fv[k].add(dvW * fvb);
                        ff[k].add(dvW * (float)s.row(FD_F + k)[b]);
                        fdr[k].add(dvW * (float)s.row(FD_FDRAG + k)[b]);
                    }
                    fvel[0].add(dvW * vb.x);
                    fvel[1].add(dvW * vb.y);
                    fvel[2].add(dvW * vb.z);
                    por.add(dvW * xb.z);
                    fdens.add(Wab * mb);
                    sum.add(dvW);
                }
            }
    const double ma = s.row(FD_MASS)[a];
    double f[3] = {0, 0, 0}, fpv[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) {
        f[d] = s.row(FD_F + d)[a];
        fpv[d] = s.row(FD_FP + d)[a];
    }
    const double ssum = (double)sum.s - (double)sum.c;
    double pr = (double)por.s - (double)por.c;
    double vel[3], fdrag_out[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) vel[k] = (double)fvel[k].s - (double)fvel[k].c;
    if (ssum > 0.5) {
        const double rsum = 1.0 / ssum;
        double fpfbd[3], fvd[3];
        for (int k = 0; k < c.nd; k++) {
            fpfbd[k] = ((double)fpfb[k].s - (double)fpfb[k].c) * rsum;
            fvd[k] = ((double)fv[k].s - (double)fv[k].c) * rsum;
            vel[k] *= rsum;
            s.row(FD_FB + k)[a] = fpfbd[k];
            s.row(FD_FV + k)[a] = fvd[k];
        }
        pr *= rsum;
        /* Di Felice drag (sph.h:1575-1631), per particle in FP64 */
        double dv[3] = {0, 0, 0}, vd2 = 0.0;
        for (int k = 0; k < c.nd; k++) {
            dv[k] = pr * (vel[k] - s.row(FD_VHAT + k)[a]);
            vd2 += dv[k] * dv[k];
        }
        const double vdiff = sqrt(vd2);
        double fdv[3] = {0, 0, 0};
        if (vdiff != 0) {
            const double A = c.pi * (c.dem_radius * c.dem_radius);
            const double Re = (2.0 * c.dem_radius / c.viscosity) * vdiff;
            const double lg = 1.5 - log10(Re);
            const double dragGamma = 3.7 - 0.65 * exp(-(lg * lg) / 2.0);
            const double cc0 = 0.63 + 4.8 / sqrt(Re);
            const double sc = 0.5 * A * (cc0 * cc0) * vdiff;
            const double pw = pow(pr, -dragGamma);
            for (int k = 0; k < c.nd; k++) fdv[k] = sc * dv[k] * pw;
        }
        for (int k = 0; k < c.nd; k++) {
            fdrag_out[k] = (c.dem_vol / ma) * (fvd[k] + fpfbd[k]) + (c.dens / ma) * fdv[k];
            f[k] += fdrag_out[k];
        }
    }
    for (int k = 0; k < 3; k++) {
        s.row(FD_FVEL + k)[a] = vel[k];
        s.row(FD_FDRAG + k)[a] = fdrag_out[k];
    }
    s.row(FD_POR)[a] = pr;
    s.row(FD_SHEP)[a] = ssum;
    /* DEM contacts over the DEM grid */
    const CellCoord cd = dem_cell_of(c, ra);
    const float4 pa = P0[a];
    const Grid32 GD = dem_grid32(c, g);
    const double Ra = s.row(FD_RADIUS)[a] > 0 ? s.row(FD_RADIUS)[a] : c.dem_radius;
    double fc64[3] = {0, 0, 0};
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
            for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cd, ox, oy, oz, GD.dims, c.periodic, c.nd, sh);
                if (lin < 0) continue;
                const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
                for (int b = start[GD.n_sph_cells + lin]; b < start[GD.n_sph_cells + lin + 1]; b++) {
                    if (b == a && !shifted) continue;
                    if ((tg[b] & 0xff) != T_DEM) continue;
                    const float4 pb = P0[b];
                    const float dx = pa.x - pb.x - ox * GD.cell[0], dy = pa.y - pb.y - oy * GD.cell[1],
                                dz = pa.z - pb.z - oz * GD.cell[2];
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    const float t = 2.f * fmaxf(ha, pb.w);
                    const float T = t * t;
                    if (r2 > T * (1.f + 4e-6f)) continue;
                    if (r2 >= T * (1.f - 4e-6f) && !exact_pair(c, s, (int)a, b, sh, 0.0, false)) continue;
                    if (shifted && !image_exists(tg[b] >> 8, sh, c.nd)) continue;
                    const double Rb = s.row(FD_RADIUS)[b] > 0 ? s.row(FD_RADIUS)[b] : c.dem_radius;
                    if ((float)(Ra + Rb) * 1.0001f - sqrtf(r2) <= 0.f) continue;
                    /* a contact: overlap = 2R - r cancels, so take r and the
                     * force in FP64 (a few contacts per particle) */
                    double dd[3] = {0, 0, 0};
                    for (int k = 0; k < c.nd; k++)
                        dd[k] = ra[k] - image_pos(s.row(FD_R + k)[b], sh[k], c.rmin[k], c.rmax[k]);
                    const double r = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                    const double overlap = (Ra + Rb) - r;
                    if (overlap > 0.0) {
                        double nrm[3] = {0, 0, 0}, od = 0.0;
                        for (int k = 0; k < c.nd; k++) {
                            nrm[k] = dd[k] / r;
                            od -= (s.row(FD_VHAT + k)[a] - s.row(FD_VHAT + k)[b]) * nrm[k];
                        }
                        const double sN = c.dem_k * overlap + c.dem_gamma * od;
                        for (int k = 0; k < c.nd; k++) fc64[k] += (sN * nrm[k]) / ma;
                    }
                }
            }
    for (int k = 0; k < c.nd; k++) {
        s.row(FD_F + k)[a] = f[k] + fc64[k];
        s.row(FD_FP + k)[a] = fpv[k] + fc64[k];
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
        cnt[tag] = m;
        return;
    }
    for (int j = 0; j < m; j++) idx[offs[tag] + j] = s.irow(FI_TAG)[nbr[(int64_t)j * ld + a] & B_MASK];
}

}  // namespace

void mixed_list_export(sphdem_ctx *c, int *cnt, const long long *offs, int *idx) {
    k_list_export<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->mx_tg, c->mx_nbr, c->mx_ncnt, c->cap, c->n,
                                                              cnt, offs, idx);
}

/* ---------------------------------------------------------------------- */
namespace mixed {

void pack(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "pack32", k_pack, grid_for(c->n, 256), 256, 0, c->cfg, c->A, c->buf.skey, c->g, c->mx_pos,
                  c->mx_vel, c->mx_aux, c->mx_tg, c->n);
}
void nlist(sphdem_ctx *c) {
    const int blocks = std::max(1, std::min(1 << 16, (c->cfg.sph_cells_cap + 3) / 4));
    SPHDEM_LAUNCH(c, "nlist32", k_nlist, blocks, BLK, 0, c->cfg, c->A, c->buf.start, c->g, c->mx_pos, c->mx_tg,
                  c->mx_nbr, c->mx_ncnt, c->mx_maxn, c->cap, 0);
}

/* largest neighbour count at the current positions (sizes the lists) */
int nlist_max_count(sphdem_ctx *c) {
    const int blocks = std::max(1, std::min(1 << 16, (c->cfg.sph_cells_cap + 3) / 4));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(c->mx_ncnt, 0, c->n * sizeof(int), c->stream));
    k_nlist<<<blocks, BLK, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, c->mx_pos, c->mx_tg, c->mx_nbr,
                                           c->mx_ncnt, 0, c->cap, 1);
    std::vector<int> h(c->n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(h.data(), c->mx_ncnt, c->n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    int m = 0;
    for (int v : h) m = std::max(m, v);
    return m;
}
void omega_eos(sphdem_ctx *c, bool omega, bool eos) {
    SPHDEM_LAUNCH(c, omega ? "omega_eos32" : "eos32", k_omega_eos32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g,
                  c->mx_pos, c->mx_vel, c->mx_aux, c->mx_tg, c->mx_nbr, c->mx_ncnt, c->cap, c->n, (int)omega,
                  (int)eos, c->mx_om);
}
void force(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "force32", k_force32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->mx_pos, c->mx_vel,
                  c->mx_aux, c->mx_om, c->mx_tg, c->mx_nbr, c->mx_ncnt, c->cap, c->n);
}
void dddt(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dddt32", k_dddt32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->mx_pos, c->mx_vel,
                  c->mx_aux, c->mx_om, c->mx_tg, c->mx_nbr, c->mx_ncnt, c->cap, c->n);
}
void porosity(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "porosity32", k_porosity32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g,
                  c->mx_pos, c->mx_vel, c->mx_tg, c->n);
}
void dem_drag(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_drag32", k_dem_drag32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g,
                  c->mx_pos, c->mx_tg, c->n);
}
void dem_end(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_end32", k_dem_end32, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g,
                  c->mx_pos, c->mx_vel, c->mx_aux, c->mx_tg, c->n);
}

}  // namespace mixed
}  // namespace sphdem
