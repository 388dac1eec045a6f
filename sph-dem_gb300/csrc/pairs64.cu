/*
 * FP64 pair passes: the reference arithmetic of every neighbour functor of
 * the hot path, one thread per target particle over the sorted bucket lists.
 *
 *   k_porosity  calcPorosity + calcShepSum        sph.h:1323-1341, 1303-1320
 *   k_dem_drag  calcDEMtoSPHDrag + finalisePorosity + setPorosityForBoundary
 *                                                 sph.h:1343-1362, 1289-1296, 1263-1265
 *   k_omega_eos calcOmega + calcPressSpsoundPdr2   sph.h:438-451, sphIncompress.h:863-896
 *   k_force     calcForce (calcViscForce, calcPressForce, calcNormal,
 *               calcBoundaryForces) + the Courant / viscous / accel dt
 *               conditions                        sphIncompress.h:899-972, sph.h:545-918
 *   k_dddt      calcDddtDudt                      sphIncompress.h:783-851
 *   k_dem_end   calcFPI + calcParticleDrag + calcDEMContacts
 *                                                 sph.h:1708-1792, 1575-1631, 1676-1706
 *   k_invm      calcInvM + inverseSym (CORRECTED_GRADIENT)
 *                                                 sph.h:393-434, vect.h:49-111
 *   k_reinit_h, k_reinit_dens
 *               the density re-initialisation of start(): ten rounds of
 *               calcHFromDens + calcDensity       sphIncompress.cpp:19-35,
 *                                                 sph.h:1823-1825, 1172-1184
 *
 * Neighbour sets are those of the reference exactly: the same 3^d bucket
 * stencil, the FP64 predicate |r_a-r_b|^2 <= (2 max(h_a,h_b))^2 evaluated
 * without FMA in blitz's order, periodic images only where the reference
 * holds a ghost copy, and the asymmetric SPH->DEM bucket rule of
 * dataLL.cpp:1154-1190.  Within a bucket, neighbours are visited in tag
 * order, which is the reference's own order for non-periodic cases.
 *
 * The Shepard sum is the only scatter of the reference (SPH particles add
 * into their DEM neighbours); it stays a scatter here with FP64 atomics.
 *
 * Roofline: FP64-pipe-bound (this GPU's FP64 rate is a small fraction of
 * its FP32 rate); this path is the plain-FP64 baseline.
 */
#include <cfloat>

#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 128;

__device__ __forceinline__ double dot3(const double *a, const double *b, int nd) {
    if (nd == 3) return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
    if (nd == 2) return a[0] * b[0] + a[1] * b[1];
    return a[0] * b[0];
}

/* Wendland C2 pieces (sph.h:74-80, 136-142, 199-205): K and dK/dq */
__device__ __forceinline__ double wK(double q, double wcon) {
    if (q > 2.0) return 0.0;
    const double t = 2.0 - q, t2 = t * t;
    return wcon * (t2 * t2) * (1.0 + 2.0 * q);
}
__device__ __forceinline__ double wdK(double q, double wcon) {
    if (q > 2.0) return 0.0;
    const double t = 2.0 - q, t2 = t * t;
    return wcon * (-4 * (t2 * t) * (1 + 2 * q) + 2 * (t2 * t2));
}

/* the displacement r_a - image(r_b) and the exact neighbour predicate */
__device__ __forceinline__ bool pair_geom(const DevCfg &c, const DevState &s, int b, const int *sh,
                                          const double *ra, double ha, double *dx, double &r2) {
    for (int d = 0; d < 3; d++) dx[d] = 0.0;
    for (int d = 0; d < c.nd; d++)
        dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
    r2 = exact_len2(dx, c.nd);
    const double hb = s.row(FD_H)[b];
    const double t = 2.0 * (ha > hb ? ha : hb);
    if (r2 > dmul(t, t)) return false;
    if ((sh[0] | sh[1] | sh[2]) && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return false;
    return true;
}

__device__ __forceinline__ void block_min_atomic(double v, unsigned long long *target) {
    __shared__ double smin[32];
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) smin[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? smin[lane] : DBL_MAX;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v < DBL_MAX) atomic_min_pos(target, v);
    }
}

/* ---------------------------------------------------------------------- */
/* SPH -> DEM coupling search (calcNeighboursCoupling for non-DEM particles) */
template <class Body>
__device__ __forceinline__ void scan_coupling(const DevCfg &c, const DevState &s, const int *start,
                                              int dem_base, const double *ra, Body &&body) {
    int cs[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) cs[d] = ref_dem_cell(ra[d], c, d);
    const CellCoord cc = dem_cell_of(c, ra);
    scan_cells(cc, c.ddims, c.periodic, c.nd, start, dem_base, [&](int b, const int *sh) {
        if (s.irow(FI_IAM)[b] != T_DEM) return;
        int cd[3] = {0, 0, 0};
        double rb[3] = {0, 0, 0};
        const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
        for (int d = 0; d < c.nd; d++) {
            rb[d] = image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]);
            cd[d] = shifted ? ref_dem_cell(rb[d], c, d) : s.irow(FI_RDC0 + d)[b];
        }
        if (!coupling_rule(cs, cd, c)) return;
        double dx[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) dx[d] = dsub(ra[d], rb[d]);
        const double r2 = exact_len2(dx, c.nd);
        if (!(r2 < c.rc2)) return;  /* beyond Rc every contribution is exactly 0 */
        if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return;
        body(b, dx, r2);
    });
}

__global__ void k_porosity(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const int dem_base = g->n_sph_cells;
    double ra[3] = {0, 0, 0}, va[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) {
        ra[d] = s.row(FD_R + d)[a];
        va[d] = s.row(FD_VHAT + d)[a];
    }
    const double dvol = s.row(FD_MASS)[a] / s.row(FD_DENS)[a];
    double por = 0.0, dpordt = 0.0, gp[3] = {0, 0, 0};
    scan_coupling(c, s, start, dem_base, ra, [&](int b, const double *dx, double r2) {
        const double r = sqrt(r2);
        const double q = r * c.two_over_rc;
        const double Wa = c.c_ihn * wK(q, c.wcon);
        por += c.por_incr * Wa;
        if (r != 0.0) {
            double dv[3] = {0, 0, 0};
            for (int d = 0; d < c.nd; d++) dv[d] = va[d] - s.row(FD_VHAT + d)[b];
            const double Fq = c.c_ihn2 * wdK(q, c.wcon) / q;
            dpordt -= c.dem_vol * dot3(dv, dx, c.nd) * Fq;
            for (int d = 0; d < c.nd; d++) gp[d] += c.dem_vol * dx[d] * Fq;
        }
        atomicAdd(&s.row(FD_SHEP)[b], dvol * Wa);
    });
    s.row(FD_POR)[a] = por;
    s.row(FD_DPORDT)[a] = dpordt;
    for (int d = 0; d < 3; d++) s.row(FD_GPOR + d)[a] = gp[d];
}

__global__ void k_zero_dem_shep(DevState s, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (s.irow(FI_IAM)[i] == T_DEM) s.row(FD_SHEP)[i] = 0.0;
}

__global__ void k_dem_drag(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int t = s.irow(FI_IAM)[a];
    if (is_boundary(t)) {
        s.row(FD_POR)[a] = 1.0;
        return;
    }
    if (!is_sph_or_sphb(t)) return;
    const int dem_base = g->n_sph_cells;
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double densa = s.row(FD_DENS)[a];
    const double rdens = c.nd == 2 ? (1.0 / (2.0 * c.dem_radius)) / densa : 1.0 / densa;
    double fd[3] = {0, 0, 0};
    scan_coupling(c, s, start, dem_base, ra, [&](int b, const double *dx, double r2) {
        const double r = sqrt(r2);
        const double w = c.c_ihn * wK(r * c.two_over_rc, c.wcon);
        const double mb = s.row(FD_MASS)[b], sb = s.row(FD_SHEP)[b];
        for (int d = 0; d < c.nd; d++) fd[d] -= mb * rdens * s.row(FD_FDRAG + d)[b] * w / sb;
    });
    for (int d = 0; d < c.nd; d++) {
        s.row(FD_FDRAG + d)[a] = fd[d];
        s.row(FD_F + d)[a] += fd[d];
    }
    double por = 1.0 - s.row(FD_POR)[a];
    if (por < 0.37) {
        por = 0.37;
        s.row(FD_DPORDT)[a] = 0.0;
        for (int d = 0; d < 3; d++) s.row(FD_GPOR + d)[a] = 0.0;
    }
    s.row(FD_POR)[a] = por;
}

/* ---------------------------------------------------------------------- */
__global__ void k_omega_eos(DevCfg c, DevState s, const int *start, const int *skey,
                            const DevGlobals *g, int64_t n, int do_omega, int do_eos) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const GridInfo gi = load_grid(g);
    const double ha = s.row(FD_H)[a], densa = s.row(FD_DENS)[a];
    if (do_omega) {
        double ra[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
        const double iha = s.row(FD_IH)[a], ihna = s.row(FD_IHN)[a];
        const double pd_coef = c.nd * (ihna * iha);  /* NDIM/pow(h,NDIM+1) */
        /* pdWh(q,h) = ihn*pdKh - nd/h^(nd+1)*K, pdKh = -q*dK/dq/h  (sph.h:285-312) */
        double om = s.row(FD_MASS)[a] * (ihna * (-0.0) - pd_coef * wK(0.0, c.wcon));
        const CellCoord cc = decode_cell(skey[a], gi.sdims, c.nd);
        scan_cells(cc, gi.sdims, c.periodic, c.nd, start, 0, [&](int b, const int *sh) {
            if (b == a && !(sh[0] | sh[1] | sh[2])) return;
            double dx[3], r2;
            if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
            if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) return;
            const double q = sqrt(r2) * iha;
            const double pdkh = -q * wdK(q, c.wcon) * iha;
            om += s.row(FD_MASS)[b] * (ihna * pdkh - pd_coef * wK(q, c.wcon));
        });
        s.row(FD_OMEGA)[a] = 1 + ha * om / (densa * c.nd);
    }
    if (do_eos) {
        double press;
        double x = c.liq_dem() ? densa / (c.refd * s.row(FD_POR)[a]) : densa / c.refd;
        if (!c.liq_dem() || c.gamma == 7.0) {
            const double x2 = x * x;
            press = c.prb * (x2 * x2 * x2 * x - 1.0);
        } else {
            press = c.prb * (pow(x, c.gamma) - 1.0);
        }
        s.row(FD_PRESS)[a] = press;
        s.row(FD_PDR2)[a] = press / (densa * densa);
    }
}

/* ---------------------------------------------------------------------- */
/* calcNormal, sph.h:736-779 */
__device__ __forceinline__ void calc_normal(const DevCfg &c, const DevState &s, int b, const double *dx, double r,
                                            double *normp, double *normt) {
    double n1[3] = {0, 0, 0}, n2[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) {
        n1[d] = s.row(FD_N1 + d)[b];
        n2[d] = s.row(FD_N2 + d)[b];
        normt[d] = c.nd == 3 ? s.row(FD_N3 + d)[b] : 0.0;
    }
    const bool n2zero = n2[0] == 0 && n2[1] == 0 && n2[2] == 0;
    if (n2zero) {
        for (int d = 0; d < 3; d++) normp[d] = n1[d];
        return;
    }
    const float rdot1 = dot3(dx, n1, c.nd);
    const float rdot2 = dot3(dx, n2, c.nd);
    const float rntest = r * r * dot3(n1, n2, c.nd) - rdot1 * rdot2;
    if (rntest <= 0) {
        for (int d = 0; d < c.nd; d++) normp[d] = dx[d] / r;
        return;
    }
    const int con = s.irow(FI_CONCAVE)[b] ? 1 : -1;
    if (con * (rdot1 - rdot2) > 0)
        for (int d = 0; d < 3; d++) normp[d] = n1[d];
    else
        for (int d = 0; d < 3; d++) normp[d] = n2[d];
}

/* ---------------------------------------------------------------------- */
/* CORRECTED_GRADIENT: per sph / sphBoundary particle, rows CG_M.. of the
 * matrix invM (nd x nd, row-major), CG_C.. of sumGrad/sum and CG_S of sum */
struct CgRow {
    double m[9], cs[3], sum;
};

__device__ __forceinline__ void cg_load(const double *cg, int64_t cap, int64_t a, int nd, CgRow &o) {
    for (int k = 0; k < nd * nd; k++) o.m[k] = cg[(CG_M + k) * cap + a];
    for (int d = 0; d < nd; d++) o.cs[d] = cg[(CG_C + d) * cap + a];
    o.sum = cg[CG_S * cap + a];
}

/* gradW with CORRECTED_GRADIENT (sph.h:325-326): invM ((dr F - sumGrad/sum)/sum),
 * the product row by row from 0 (vect.h:39-47) */
__device__ __forceinline__ void cg_apply(const CgRow &w, const double *dx, double F, int nd, double *out) {
    double t[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) t[d] = (dx[d] * F - w.cs[d]) / w.sum;
    for (int i = 0; i < nd; i++) {
        double v = 0.0;
        for (int j = 0; j < nd; j++) v += w.m[i * nd + j] * t[j];
        out[i] = v;
    }
}

/* inverseSym (vect.h:49-111): adjugate over determinant; identity when the
 * determinant is 0.  1D (which the reference does not define) inverts the
 * scalar. */
__device__ void inverse_sym(double *a, int nd) {
    if (nd == 1) {
        a[0] = a[0] != 0.0 ? 1.0 / a[0] : 1.0;
        return;
    }
    if (nd == 2) {
        const double A = a[0], B = a[1], C = a[2], D = a[3];
        const double det = dsub(dmul(A, D), dmul(B, C));
        if (det != 0.0) {
            a[0] = D / det;
            a[1] = -B / det;
            a[2] = -C / det;
            a[3] = A / det;
        } else {
            a[0] = 1.0;
            a[1] = 0.0;
            a[2] = 0.0;
            a[3] = 1.0;
        }
        return;
    }
    const double A0 = a[0], B0 = a[1], C0 = a[2], D0 = a[3], E0 = a[4], F0 = a[5], G0 = a[6], H0 = a[7], K0 = a[8];
    const double cA = dsub(dmul(E0, K0), dmul(F0, H0)), cB = dsub(dmul(F0, G0), dmul(D0, K0));
    const double cC = dsub(dmul(D0, H0), dmul(E0, G0)), cD = dsub(dmul(C0, H0), dmul(B0, K0));
    const double cE = dsub(dmul(A0, K0), dmul(C0, G0)), cF = dsub(dmul(B0, G0), dmul(A0, H0));
    const double cG = dsub(dmul(B0, F0), dmul(C0, E0)), cH = dsub(dmul(C0, D0), dmul(A0, F0));
    const double cK = dsub(dmul(A0, E0), dmul(B0, D0));
    const double Z = dadd(dadd(dmul(A0, cA), dmul(B0, dsub(dmul(F0, G0), dmul(K0, D0)))), dmul(C0, cC));
    if (Z != 0.0) {
        const double o[9] = {cA, cD, cG, cB, cE, cH, cC, cF, cK};
        for (int k = 0; k < 9; k++) a[k] = o[k] / Z;
    } else {
        for (int k = 0; k < 9; k++) a[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
}

/* calcInvM (sph.h:393-434) of every sph / sphBoundary particle over the
 * neighbours of the last rebuild: sum = (m/rho) W(0,h) + sum dvol W(r/hav,hav),
 * sumGrad = sum dvol dr F(r/hav,hav), M = -sum dvol (dr F - sumGrad/sum)/sum (x) dr,
 * invM = M^-1 (identity without neighbours) */
__global__ void k_invm(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g, double *cg,
                       int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const GridInfo gi = load_grid(g);
    const int nd = c.nd;
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ha = s.row(FD_H)[a];
    double sum = (s.row(FD_MASS)[a] / s.row(FD_DENS)[a]) * (s.row(FD_IHN)[a] * wK(0.0, c.wcon));
    double sg[3] = {0, 0, 0}, m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int nn = 0;
    const CellCoord cc = decode_cell(skey[a], gi.sdims, nd);
    /* F(q, hav) and W(q, hav) of a pair (sph.h:74-80, 306-308) */
    auto kern = [&](double r, double hb, double &F, double &W) {
        const double hav = 0.5 * (ha + hb);
        const double q = r / hav, ih = 1.0 / hav;
        double ihn = ih;
        for (int d = 1; d < nd; d++) ihn *= ih;
        F = (ihn * ih * ih) * wdK(q, c.wcon) / q;
        W = ihn * wK(q, c.wcon);
    };
    scan_cells(cc, gi.sdims, c.periodic, nd, start, 0, [&](int b, const int *sh) {
        if (b == a && !(sh[0] | sh[1] | sh[2])) return;
        double dx[3], r2;
        if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
        nn++;
        if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) return;
        const double dvol = s.row(FD_MASS)[b] / s.row(FD_DENS)[b];
        double F, W;
        kern(sqrt(r2), s.row(FD_H)[b], F, W);
        sum += dvol * W;
        for (int d = 0; d < nd; d++) sg[d] += (dvol * dx[d]) * F;
    });
    if (nn == 0) {
        for (int i = 0; i < nd; i++) m[i * nd + i] = 1.0;
    } else {
        scan_cells(cc, gi.sdims, c.periodic, nd, start, 0, [&](int b, const int *sh) {
            if (b == a && !(sh[0] | sh[1] | sh[2])) return;
            double dx[3], r2;
            if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
            if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) return;
            const double dvol = s.row(FD_MASS)[b] / s.row(FD_DENS)[b];
            double F, W;
            kern(sqrt(r2), s.row(FD_H)[b], F, W);
            double gw[3] = {0, 0, 0};
            for (int d = 0; d < nd; d++) gw[d] = (dx[d] * F - sg[d] / sum) / sum;
            for (int i = 0; i < nd; i++)
                for (int j = 0; j < nd; j++) m[i * nd + j] -= dvol * dmul(gw[i], dx[j]);
        });
        inverse_sym(m, nd);
    }
    const int64_t cap = s.cap;
    for (int k = 0; k < nd * nd; k++) cg[(CG_M + k) * cap + a] = m[k];
    for (int d = 0; d < nd; d++) cg[(CG_C + d) * cap + a] = sg[d] / sum;
    cg[CG_S * cap + a] = sum;
}

/* ---------------------------------------------------------------------- */
/* Density re-initialisation (sphIncompress.cpp:19-35).  The neighbour lists
 * of the reference are built lazily after the first calcHFromDens, so the
 * neighbour predicate uses that first h (kept in hp) through all ten
 * rounds, while calcDensity uses each round's own h. */
__global__ void k_reinit_h(DevCfg c, DevState s, double *hp, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const double m = s.row(FD_MASS)[a], rho = s.row(FD_DENS)[a];
    const double x = c.precision == SPHDEM_PREC_MIXED ? m * recip(c, rho) : m / rho;
    const double h = smoothing_length(c, x);
    s.row(FD_H)[a] = h;
    hp[a] = h;
}

__global__ void k_reinit_dens(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g,
                              const double *hp, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const GridInfo gi = load_grid(g);
    const int nd = c.nd;
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ma = s.row(FD_MASS)[a], hpa = hp[a];
    double h = s.row(FD_H)[a], rho = s.row(FD_DENS)[a];
    const CellCoord cc = decode_cell(skey[a], gi.sdims, nd);
    for (int round = 0; round < 10; round++) {
        if (round > 0) {
            const double x = c.precision == SPHDEM_PREC_MIXED ? ma * recip(c, rho) : ma / rho;
            h = smoothing_length(c, x);
        }
        const double ih = recip(c, h);
        double ihn = ih;
        for (int d = 1; d < nd; d++) ihn *= ih;
        double sum = ma * (ihn * wK(0.0, c.wcon));
        scan_cells(cc, gi.sdims, c.periodic, nd, start, 0, [&](int b, const int *sh) {
            const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
            if (b == a && !shifted) return;
            if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) return;
            double dx[3] = {0, 0, 0};
            for (int d = 0; d < nd; d++)
                dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
            const double r2 = exact_len2(dx, nd);
            const double hb = hp[b];
            const double t = 2.0 * (hpa > hb ? hpa : hb);
            if (r2 > dmul(t, t)) return;
            if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, nd)) return;
            const double q = c.precision == SPHDEM_PREC_MIXED ? sqrt(r2) * ih : sqrt(r2) / h;
            sum += s.row(FD_MASS)[b] * (ihn * wK(q, c.wcon));
        });
        rho = sum;
    }
    s.row(FD_H)[a] = h;
    h_derived(c, s, a);
    s.row(FD_DENS)[a] = rho;
}

__global__ void k_force(DevCfg c, DevState s, const int *start, const int *skey, DevGlobals *g, const double *cg,
                        int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double ndt = DBL_MAX;
    if (a < n && is_sph_or_sphb(s.irow(FI_IAM)[a])) {
        const GridInfo gi = load_grid(g);
        const int ta = s.irow(FI_IAM)[a];
        double ra[3] = {0, 0, 0}, va[3] = {0, 0, 0};
        double f[3] = {0, 0, 0}, fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, fb[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) {
            ra[d] = s.row(FD_R + d)[a];
            va[d] = s.row(FD_VHAT + d)[a];
            f[d] = s.row(FD_F + d)[a];
            fp[d] = s.row(FD_FP + d)[a];
            fv[d] = s.row(FD_FV + d)[a];
            fb[d] = s.row(FD_FB + d)[a];
        }
        const double ha = s.row(FD_H)[a], iha = s.row(FD_IH)[a], ihn2a = s.row(FD_IHN2)[a];
        const double densa = s.row(FD_DENS)[a], pdr2a = s.row(FD_PDR2)[a], ma = s.row(FD_MASS)[a];
        const double oma = c.var_h() ? s.row(FD_OMEGA)[a] : 1.0;
        const bool no_anti = c.flags & SPHDEM_F_NO_ANTICLUMPING;
        CgRow cw;
        if (cg) cg_load(cg, s.cap, a, c.nd, cw);
        const CellCoord cc = decode_cell(skey[a], gi.sdims, c.nd);
        scan_cells(cc, gi.sdims, c.periodic, c.nd, start, 0, [&](int b, const int *sh) {
            if (b == a && !(sh[0] | sh[1] | sh[2])) return;
            double dx[3], r2;
            if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
            const int tb = s.irow(FI_IAM)[b];
            const double r = sqrt(r2);
            const double hb = s.row(FD_H)[b], ihb = s.row(FD_IH)[b], ihn2b = s.row(FD_IHN2)[b];
            const double qa = r * iha, qb = r * ihb;
            /* gradW (sph.h:322-342): dr*F(q,h), F = ihn2*dK/dq/q; /omega_a with VAR_H */
            double Fa = 0.0, Fb = 0.0;
            if (qa != 0) Fa = ihn2a * wdK(qa, c.wcon) / qa;
            if (qb != 0) Fb = ihn2b * wdK(qb, c.wcon) / qb;
            double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
            double wa[3] = {0, 0, 0}, wb[3] = {0, 0, 0};
            if (cg) {
                cg_apply(cw, dx, Fa, c.nd, wa);
                cg_apply(cw, dx, Fb, c.nd, wb);
            } else {
                for (int d = 0; d < c.nd; d++) {
                    wa[d] = dx[d] * Fa;
                    wb[d] = dx[d] * Fb;
                }
            }
            for (int d = 0; d < c.nd; d++) {
                if (c.var_h()) {
                    gA[d] = wa[d] / oma;
                    gB[d] = wb[d] / oma;
                } else {
                    gA[d] = gB[d] = 0.5 * (wa[d] + wb[d]);
                }
            }
            const double densb = s.row(FD_DENS)[b], mb = s.row(FD_MASS)[b];
            const double hav = 0.5 * (ha + hb);
            if (ta == T_SPH && tb != T_DEM && tb != T_DEMB) {
                /* calcViscForce, sph.h:579-666 */
                double dv[3] = {0, 0, 0}, gm[3] = {0, 0, 0};
                for (int d = 0; d < c.nd; d++) {
                    dv[d] = va[d] - s.row(FD_VHAT + d)[b];
                    gm[d] = 0.5 * (gA[d] + gB[d]);
                }
                const double vdr = dot3(dx, dv, c.nd);
                double fvp[3] = {0, 0, 0};
                double vsig = 0.0;
                if (c.visc == SPHDEM_VISC_MORRIS) {
                    double visc = c.viscosity * (densa + densb) / (densa * densb);
                    vsig = 2.0 * c.spsound;
                    if (c.liq_dem()) visc = 2.0 * c.viscosity * c.dens / (densa * densb);
                    const double dg = dot3(dx, gm, c.nd);
                    const double den = r * r + 0.01 * (hav * hav);
                    for (int d = 0; d < c.nd; d++) fvp[d] = dv[d] * mb * visc * dg / den;
                } else if (c.visc == SPHDEM_VISC_MONAGHAN) {
                    const double rr = r != 0.0 ? 1 / r : 0.0;
                    const double viss = vdr * rr;
                    if (!c.liq_dem()) vsig = 2.0 * c.spsound + 2.0 * fabs(viss);
                    const double visc = viss * vsig * c.alpha_mon / (densa + densb);
                    for (int d = 0; d < c.nd; d++) fvp[d] = mb * visc * gm[d];
                } else if (c.visc == SPHDEM_VISC_ARTIFICIAL) {
                    double avsig = 0.0, avisc = 0.0;
                    if (vdr < 0) {
                        const double rr = r != 0.0 ? 1 / r : 0.0;
                        const double viss = vdr * rr;
                        avsig = 2.0 * c.spsound - 4.0 * viss;
                        avisc = viss * avsig * c.alpha_art / (densa + densb);
                    }
                    for (int d = 0; d < c.nd; d++) f[d] += mb * avisc * gm[d];
                    vsig = fmax(vsig, avsig);
                }
                ndt = fmin(ndt, 0.6 * hav / vsig);
                const double vdc = c.visc == SPHDEM_VISC_MONAGHAN ? 0.06 : 0.125;
                ndt = fmin(ndt, vdc * (hav * hav) / c.viscosity);
                for (int d = 0; d < c.nd; d++) {
                    fv[d] += fvp[d];
                    f[d] += fvp[d];
                }
            }
            double kdwPowNeps = 0.0;
            if (!no_anti) {
                const double kdw = wK(r / hav, c.wcon) / c.k_anti;
                const double k2 = kdw * kdw;
                kdwPowNeps = k2 * k2;
            }
            if (is_boundary(tb)) {
                /* calcNormal + calcBoundaryForces, sph.h:736-918 */
                double normp[3] = {0, 0, 0}, normt[3] = {0, 0, 0};
                calc_normal(c, s, b, dx, r, normp, normt);
                double dv[3] = {0, 0, 0};
                for (int d = 0; d < c.nd; d++) dv[d] = va[d] - s.row(FD_VHAT + d)[b];
                const double rperp = dot3(normp, dx, c.nd);
                double rt[3] = {0, 0, 0};
                for (int d = 0; d < c.nd; d++) rt[d] = dx[d] - rperp * normp[d];
                double pt0, pt1;
                const double rDelP = 1.0 / (c.bfac * c.psep);
                if (c.nd == 3) {
                    pt0 = fabs(dot3(rt, normt, 3));
                    const double cr[3] = {rt[1] * normt[2] - rt[2] * normt[1], rt[2] * normt[0] - rt[0] * normt[2],
                                          rt[0] * normt[1] - rt[1] * normt[0]};
                    pt1 = sqrt(dot3(cr, cr, 3));
                } else {
                    pt0 = sqrt(dot3(rt, rt, c.nd));
                    pt1 = 0;
                }
                const double pd0 = pt0 * rDelP, pd1 = pt1 * rDelP;
                if (pd0 <= 1.0 && pd1 <= 1.0) {
                    const double pesky = 0.25 * (1 + cos(c.pi * pd0)) * (1 + cos(c.pi * pd1));
                    const double q = fabs(rperp) / (1.0 * c.psep);
                    double fbp[3] = {0, 0, 0};
                    if (q < 2.0) {
                        const int beta = dot3(dx, dv, c.nd) < 0 ? 1 : 0;
                        const double bigA = 0.01 * (c.spsound * c.spsound) - beta * c.spsound * dot3(dv, normp, c.nd);
                        const double bfact = 1.0 / fabs(rperp);
                        const double QIN = 2.0 / 3.0;
                        double bforce = 0.0;
                        if (q <= QIN) bforce = bfact * QIN;
                        else if (q <= 1.0) bforce = bfact * (2.0 * q - 1.5 * q * q);
                        else if (q <= 2.0) bforce = bfact * 0.5 * ((2.0 - q) * (2.0 - q));
                        const double bigR = bigA * bforce;
                        const double amassrat = 2.0 * ma / (ma + mb);
                        const int sign = rperp < 0 ? -1 : 1;
                        for (int d = 0; d < c.nd; d++) fbp[d] = sign * amassrat * normp[d] * bigR * pesky * 1.0;
                    }
                    for (int d = 0; d < c.nd; d++) {
                        fb[d] += fbp[d];
                        f[d] += fbp[d];
                    }
                }
            } else if (tb == T_SPH || tb == T_SPHB) {
                /* calcPressForce, sph.h:692-734 */
                const double pdr2b = s.row(FD_PDR2)[b];
                const double antic = 0.01 * fabs(pdr2a + pdr2b) * kdwPowNeps;
                for (int d = 0; d < c.nd; d++) {
                    const double prfac = (pdr2a * gA[d] + pdr2b * gB[d]) + antic;
                    const double fpp = -mb * prfac;
                    fp[d] += fpp;
                    f[d] += fpp;
                }
            }
        });
        for (int d = 0; d < c.nd; d++) {
            s.row(FD_F + d)[a] = f[d];
            s.row(FD_FP + d)[a] = fp[d];
            s.row(FD_FV + d)[a] = fv[d];
            s.row(FD_FB + d)[a] = fb[d];
        }
        /* accelCondition, sph.h:566-568 */
        ndt = fmin(ndt, 0.25 * sqrt(ha / sqrt(dot3(f, f, c.nd))));
    }
    block_min_atomic(ndt, &g->new_dt_bits);
}

__global__ void k_dem_accel(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double ndt = DBL_MAX;
    if (i < n && s.irow(FI_IAM)[i] == T_DEM) {
        double f[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) f[d] = s.row(FD_F + d)[i];
        ndt = 0.25 * sqrt(s.row(FD_H)[i] / sqrt(dot3(f, f, c.nd)));
    }
    block_min_atomic(ndt, &g->new_dt_bits);
}

/* ---------------------------------------------------------------------- */
__global__ void k_dddt(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g,
                       const double *cg, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[a])) return;
    const GridInfo gi = load_grid(g);
    double ra[3] = {0, 0, 0}, va[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) {
        ra[d] = s.row(FD_R + d)[a];
        va[d] = s.row(FD_VHAT + d)[a];
    }
    const double ha = s.row(FD_H)[a], iha = s.row(FD_IH)[a], ihn2a = s.row(FD_IHN2)[a];
    const double oma = c.var_h() ? s.row(FD_OMEGA)[a] : 1.0;
    double dddt = s.row(FD_DDDT)[a];
    CgRow cw;
    if (cg) cg_load(cg, s.cap, a, c.nd, cw);
    const CellCoord cc = decode_cell(skey[a], gi.sdims, c.nd);
    scan_cells(cc, gi.sdims, c.periodic, c.nd, start, 0, [&](int b, const int *sh) {
        if (b == a && !(sh[0] | sh[1] | sh[2])) return;
        double dx[3], r2;
        if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
        const int tb = s.irow(FI_IAM)[b];
        if (is_boundary(tb) || tb == T_DEM) return;
        const double r = sqrt(r2);
        const double qa = r * iha;
        double Fa = 0.0;
        if (qa != 0) Fa = ihn2a * wdK(qa, c.wcon) / qa;
        double gw[3] = {0, 0, 0}, wa[3] = {0, 0, 0};
        if (cg) cg_apply(cw, dx, Fa, c.nd, wa);
        else
            for (int d = 0; d < c.nd; d++) wa[d] = dx[d] * Fa;
        if (c.var_h()) {
            for (int d = 0; d < c.nd; d++) gw[d] = wa[d] / oma;
        } else {
            const double qb = r * s.row(FD_IH)[b];
            double Fb = 0.0;
            if (qb != 0) Fb = s.row(FD_IHN2)[b] * wdK(qb, c.wcon) / qb;
            double wb[3] = {0, 0, 0};
            if (cg) cg_apply(cw, dx, Fb, c.nd, wb);
            else
                for (int d = 0; d < c.nd; d++) wb[d] = dx[d] * Fb;
            for (int d = 0; d < c.nd; d++) gw[d] = 0.5 * (wa[d] + wb[d]);
        }
        double dv[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) dv[d] = va[d] - s.row(FD_VHAT + d)[b];
        dddt += s.row(FD_MASS)[b] * dot3(dv, gw, c.nd);
    });
    s.row(FD_DDDT)[a] = dddt;
}

/* ---------------------------------------------------------------------- */
__device__ __forceinline__ double radius_of(const DevCfg &c, const DevState &s, int i) {
    const double r = s.row(FD_RADIUS)[i];
    return r > 0.0 ? r : c.dem_radius;
}

__global__ void k_dem_end(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    if (s.irow(FI_IAM)[a] != T_DEM) return;
    const GridInfo gi = load_grid(g);
    double ra[3] = {0, 0, 0}, va[3] = {0, 0, 0}, f[3] = {0, 0, 0}, fpv[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) {
        ra[d] = s.row(FD_R + d)[a];
        va[d] = s.row(FD_VHAT + d)[a];
        f[d] = s.row(FD_F + d)[a];
        fpv[d] = s.row(FD_FP + d)[a];
    }
    const double ha = s.row(FD_H)[a], ma = s.row(FD_MASS)[a];
    /* calcFPI over the SPH buckets (calcNeighboursCoupling for a DEM particle) */
    double sum = 0, fdens = 0, por = 0;
    double ff[3] = {0, 0, 0}, fpfb[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, fdr[3] = {0, 0, 0}, fvel[3] = {0, 0, 0};
    const CellCoord cs = sph_cell_of(c, gi, ra);
    scan_cells(cs, gi.sdims, c.periodic, c.nd, start, 0, [&](int b, const int *sh) {
        double dx[3], r2;
        if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
        if (s.irow(FI_IAM)[b] == T_BOUNDARY) return;
        const double r = sqrt(r2);
        const double mb = s.row(FD_MASS)[b];
        const double dvol = mb / s.row(FD_DENS)[b];
        const double q = r * s.row(FD_IH)[b];
        const double Wab = s.row(FD_IHN)[b] * wK(q, c.wcon);
        const double dvWab = dvol * Wab;
        for (int d = 0; d < c.nd; d++) {
            fpfb[d] += mb * Wab * (s.row(FD_FP + d)[b] + s.row(FD_FB + d)[b]);
            fv[d] += mb * Wab * s.row(FD_FV + d)[b];
            fv[d] += dvWab * s.row(FD_FV + d)[b];
            ff[d] += dvWab * s.row(FD_F + d)[b];
            fdr[d] += dvWab * s.row(FD_FDRAG + d)[b];
            fvel[d] += dvWab * s.row(FD_VHAT + d)[b];
        }
        por += dvWab * s.row(FD_POR)[b];
        fdens += Wab * mb;
        sum += dvWab;
    });
    double fdrag_out[3] = {0, 0, 0};
    if (sum > 0.5) {
        const double rsum = 1.0 / sum;
        for (int d = 0; d < c.nd; d++) {
            ff[d] *= rsum;
            fpfb[d] *= rsum;
            fv[d] *= rsum;
            fdr[d] *= rsum;
            fvel[d] *= rsum;
        }
        fdens *= rsum;
        por *= rsum;
        for (int d = 0; d < c.nd; d++) {
            s.row(FD_FB + d)[a] = fpfb[d];
            s.row(FD_FV + d)[a] = fv[d];
        }
        /* calcParticleDrag, Di Felice (sph.h:1575-1631) */
        double dv[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) dv[d] = por * (fvel[d] - va[d]);
        const double vdiff = sqrt(dot3(dv, dv, c.nd));
        double fd[3] = {0, 0, 0};
        if (vdiff != 0) {
            const double A = c.pi * (c.dem_radius * c.dem_radius);
            const double Re = (2.0 * c.dem_radius / c.viscosity) * vdiff;
            const double lg = 1.5 - log10(Re);
            const double dragGamma = 3.7 - 0.65 * exp(-(lg * lg) / 2.0);
            const double cc0 = 0.63 + 4.8 / sqrt(Re);
            const double C = cc0 * cc0;
            const double sc = (1.0 / 2.0) * A * C * vdiff;
            const double pw = pow(por, -dragGamma);
            for (int d = 0; d < c.nd; d++) fd[d] = c.drag_scale * (sc * dv[d] * pw);
        }
        for (int d = 0; d < c.nd; d++) {
            fdrag_out[d] = (c.dem_vol / ma) * (fv[d] + fpfb[d]) + (c.dens / ma) * fd[d];
            f[d] += fdrag_out[d];
        }
    } else {
        for (int d = 0; d < c.nd; d++) fvel[d] *= 1.0;  /* unnormalised, as the reference leaves it */
    }
    for (int d = 0; d < 3; d++) {
        s.row(FD_FVEL + d)[a] = fvel[d];
        s.row(FD_FDRAG + d)[a] = fdrag_out[d];
    }
    s.row(FD_POR)[a] = por;
    s.row(FD_SHEP)[a] = sum;
    /* calcDEMContacts over the DEM buckets (sph.h:1676-1706, LINEAR) */
    const double Ra = radius_of(c, s, (int)a);
    const CellCoord cd = dem_cell_of(c, ra);
    scan_cells(cd, c.ddims, c.periodic, c.nd, start, gi.n_sph_cells, [&](int b, const int *sh) {
        if (b == a && !(sh[0] | sh[1] | sh[2])) return;
        if (s.irow(FI_IAM)[b] != T_DEM) return;
        double dx[3], r2;
        if (!pair_geom(c, s, b, sh, ra, ha, dx, r2)) return;
        const double r = sqrt(r2);
        double nrm[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) {
            nrm[d] = dx[d] / r;
            dv[d] = va[d] - s.row(FD_VHAT + d)[b];
        }
        const double overlap = (Ra + radius_of(c, s, b)) - r;
        if (overlap > 0) {
            const double od = -dot3(dv, nrm, c.nd);
            const double sN = c.dem_k * overlap + c.dem_gamma * od;
            for (int d = 0; d < c.nd; d++) {
                const double fN = (sN * nrm[d]) / ma;
                fpv[d] += fN;
                f[d] += fN;
            }
        }
    });
    for (int d = 0; d < c.nd; d++) {
        s.row(FD_F + d)[a] = f[d];
        s.row(FD_FP + d)[a] = fpv[d];
    }
}

}  // namespace

void zero_dem_shep(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "zero_dem_shep", k_zero_dem_shep, grid_for(c->n, 256), 256, 0, c->A, c->n);
}
void run_porosity(sphdem_ctx *c) {
    zero_dem_shep(c);
    SPHDEM_LAUNCH(c, "porosity_fp64", k_porosity, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g, c->n);
}
void run_dem_drag(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_drag_fp64", k_dem_drag, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g, c->n);
}
void run_omega_eos(sphdem_ctx *c, bool omega, bool eos) {
    SPHDEM_LAUNCH(c, omega ? "omega_eos_fp64" : "eos_fp64", k_omega_eos, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A,
                  c->buf.start, c->buf.skey, c->g, c->n, (int)omega, (int)eos);
}
void run_force(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "force_fp64", k_force, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->buf.skey,
                  c->g, corrected_gradient(c) ? c->cg : nullptr, c->n);
}
void run_invm(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "invm_fp64", k_invm, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->buf.skey, c->g,
                  c->cg, c->n);
}
void run_reinit_density(sphdem_ctx *c) {
    rebuild(c);
    SPHDEM_LAUNCH(c, "reinit_h", k_reinit_h, grid_for(c->n, 256), 256, 0, c->cfg, c->A, c->hpred, c->n);
    SPHDEM_LAUNCH(c, "reinit_dens_fp64", k_reinit_dens, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start,
                  c->buf.skey, c->g, c->hpred, c->n);
}
void run_dem_accel(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_accel", k_dem_accel, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_dddt(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dddt_fp64", k_dddt, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->buf.skey,
                  c->g, corrected_gradient(c) ? c->cg : nullptr, c->n);
}
void run_dem_end(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_end_fp64", k_dem_end, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->buf.start, c->g, c->n);
}

}  // namespace sphdem
