/*
 * Adjoint of the coupled SPH-DEM step (reverse mode, FP64).
 *
 * Scope: LIQ_DEM handles of fluid (SPH), fixed fluid boundary (SPHB) and DEM
 * particles, Morris viscosity, constant h, no VAR_H_CORRECTION, no
 * anticlumping, gamma = 7, fixed dt, periodic axes allowed.  With hd = dt/2
 * and tag-order state (s0 before the step, s1 after), the step of
 * sphIncompress.cpp:3-251 with the sediment3D hooks reads, for a fluid
 * particle a and a DEM particle i:
 *
 *   start:   r_s = r0 + hd vh0 (all),  vh_s = vh0 + hd f0 (SPH),  rho_s = rho0 + hd dddt0
 *   middle:  e_a = sum_i V W_c(r_ai),  eps_a = max(1 - e_a, 0.37)            (calcPorosity, sph.h:1323-1341)
 *            shep_i = sum_a (m_a / rho_a) W_c(r_ai)                            (calcShepSum, sph.h:1303-1320)
 *            fd_a = -sum_i m_i fdrag0_i W_c(r_ai) / (rho_a shep_i)              (calcDEMtoSPHDrag, sph.h:1343-1362)
 *            pdr2_a = PRB((rho_a / (rho0 eps_a))^7 - 1) / rho_a^2            (sphIncompress.h:863-896)
 *            fp_a = -sum_b m_b (pdr2_a + pdr2_b) G d,  fv_a = sum_b c_ab phi(r) w_ab   (sph.h:579-734)
 *              c_ab = 2 nu rho0 m_b / (rho_a rho_b), phi = G r^2 / (r^2 + 0.01 hbar^2)
 *            f1_a = g + fd_a + fp_a + fv_a;  vh1 = vh0 + dt f1, v1 = v0 + dt f1 (SPH)
 *            DEM: r_m = r_s + hd vh0, vh_m = vh0 + hd f0
 *   end:     DEM: f_i = g + walls(r_m, vh_m) + Delta_i + contacts(r_m, vh_m)
 *              Delta_i = (V/m)(fv_i + fpfb_i) + (rho0/m) kappa Phi(por (fvel - vh_m), por)
 *              (calcFPI + calcParticleDrag, sph.h:1575-1631, 1708-1792; normalised
 *              sums over the fluid within 2 max(h): por, fpfb, fv, fvel; Delta = 0
 *              when the Shepard sum is <= 0.5), fdrag1_i = Delta_i,
 *              vh1 = vh0 + dt f, v1 = v0 + dt f
 *            fluid: r1 = r_s + hd vh1, dddt1 = continuity at r1, rho1 = rho_s + hd dddt1
 *
 * W_c(r) = C_c K(2r/Rc) is the coupling kernel, V the DEM volume increment,
 * kappa the drag scale and Phi the Di Felice law.  The reverse pass of one
 * step runs, in order: intermediates (k_cp_pre), porosity / Shepard / EOS
 * (k_cp_por), FPI + drag (k_cp_fpi), DEM walls + contacts (k_cp_dem),
 * continuity and the adjoint of f1 (k_cp_end), forces + EOS (k_cp_force),
 * porosity + DEM->fluid drag (k_cp_cpl_a), Shepard sums (k_cp_cpl_b) and the
 * adjoint of the state before the step (k_cp_assemble).  Scatters from one
 * particle kind into the other (fluid <-> DEM) are FP64 atomics; sums within
 * the fluid gather over the symmetric pair table.
 *
 * Mixed-precision handles run the two fluid pair passes (continuity and
 * forces, ~100 pairs per particle in 3D) in FP32 on double-float position
 * records with Kahan sums; the coupling passes (a few DEM partners per
 * fluid particle) stay FP64.
 *
 * Positions of the middle phase are snapshotted after it in the replay (a
 * periodic wrap in the middle rebuild would otherwise separate the
 * recomputed r_s from the frame the pair tables were built in).
 */
#include <algorithm>
#include <string>
#include <vector>

#include "adjoint.cuh"

namespace sphdem {

void PairTable::alloc(int K, int64_t n) {
    SPHDEM_CUDA_CHECK(cudaMalloc(&nb, (size_t)K * cap * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&oc, (size_t)K * n * sizeof(int2)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&cnt, (size_t)K * sizeof(int)));
}

void PairTable::free_all() {
    cudaFree(nb);
    cudaFree(oc);
    cudaFree(cnt);
    nb = nullptr;
    oc = nullptr;
    cnt = nullptr;
}

namespace {

constexpr int CB = 128;

/* accumulator slots (CP_NACC per particle) */
enum : int {
    CA_R1 = 0,      /* adjoint of the end-phase position (fluid r1, DEM r_m) */
    CA_VH1 = 3,     /* fluid: adjoint of vh1; DEM: adjoint of vh_m */
    CA_RHO = 6,     /* fluid: adjoint of rho_s (FPI) */
    CA_EPS = 7,     /* fluid: adjoint of eps (FPI) */
    CA_FP = 8,      /* fluid: adjoint of fp (FPI) */
    CA_FV = 11,     /* fluid: adjoint of fv (FPI) */
    CA_RS = 14,     /* adjoint of the middle-phase position */
    CA_FD0 = 17,    /* DEM: adjoint of the lagged drag fdrag0 */
    CA_SHEP = 20,   /* DEM: adjoint of the Shepard sum */
    CA_RHOS = 21,   /* fluid: total adjoint of rho_s */
    CA_EBAR = 22    /* fluid: adjoint of e = 1 - eps (0 where clamped) */
};
/* end-phase results (CP_NEND): total adjoint of r1, vh1, f1, fp, fv */
enum : int { CE_R1 = 0, CE_VH1 = 3, CE_F = 6, CE_P = 9, CE_V = 12 };
/* middle intermediates (CP_NMID): eps, clamped, pdr2, Shepard sum (DEM),
 * adjoint of vh_s */
enum : int { CM_EPS = 0, CM_CLAMP = 1, CM_PDR2 = 2, CM_SHEP = 3, CM_VHS = 4 };

__device__ __forceinline__ bool is_fluid(int t) { return t == T_SPH || t == T_SPHB; }

/* one warp-aggregated atomic reserves k entries per thread; every lane of
 * the warp must call it */
__device__ __forceinline__ int64_t reserve(int k, int *cnt) {
    const int lane = threadIdx.x & 31;
    int incl = k;
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

/* ---- taps: pair tables of the current buckets ------------------------ */

/* DEM particle i -> DEM in contact (neighbour predicate and positive
 * overlap), as calcDEMContacts visits them (sph.h:1676-1706) */
template <bool WRITE>
__device__ int contact_scan(const DevCfg &c, const DevState &s, const int *start, const DevGlobals *g, int64_t a,
                            int *out, int64_t room) {
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ha = s.row(FD_H)[a];
    const double Ra = s.row(FD_RADIUS)[a] > 0 ? s.row(FD_RADIUS)[a] : c.dem_radius;
    const CellCoord cd = dem_cell_of(c, ra);
    int k = 0;
    scan_cells(cd, c.ddims, c.periodic, c.nd, start, g->n_sph_cells, [&](int b, const int *sh) {
        const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
        if (b == a && !shifted) return;
        if (s.irow(FI_IAM)[b] != T_DEM) return;
        double dx[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++)
            dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
        const double r2 = exact_len2(dx, c.nd);
        const double hb = s.row(FD_H)[b];
        const double t = 2.0 * (ha > hb ? ha : hb);
        if (r2 > dmul(t, t)) return;
        if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return;
        const double Rb = s.row(FD_RADIUS)[b] > 0 ? s.row(FD_RADIUS)[b] : c.dem_radius;
        if (!((Ra + Rb) - sqrt(r2) > 0)) return;
        if (WRITE && k < room) out[k] = s.irow(FI_TAG)[b] | shift_code(sh);
        k++;
    });
    return k;
}

/* FP32 middle-phase positions of the DEM particles by state index (the tap
 * runs after the middle phase's tail drifted them by hd vhat0) */
__global__ void k_cp_dpos(DevState s, const DevGlobals *g, int64_t n, float4 *dpos) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n || s.irow(FI_IAM)[k] != T_DEM) return;
    const double hd = 0.5 * g->dt;
    float p[3];
    for (int d = 0; d < 3; d++) p[d] = (float)(s.row(FD_R + d)[k] - hd * s.row(FD_VHAT0 + d)[k]);
    dpos[k] = make_float4(p[0], p[1], p[2], 0.f);
}

/* fluid -> DEM coupling table: the bucket rule of calcNeighboursCoupling
 * (dataLL.cpp:1104-1192, asymmetric: it leaves out some pairs within Rc) as
 * the middle phase applies it, with the distance cut r < Rc as an FP32 test
 * with a relative margin of 1e-4 on Rc^2 -- a superset of the coupled pairs,
 * and pairs at or beyond Rc carry W_c = dW_c/dr = 0.  DEM positions are those
 * of the middle phase (dpos; the rule's own DEM buckets were set at its
 * rebuild). */
/* reference DEM bucket of the periodic image of DEM particle b (out of line:
 * only pairs across a periodic face take it) */
__device__ __noinline__ void image_dem_cells(const DevCfg &c, const DevState &s, int b, const int *sh, double hd,
                                             int *cd) {
    for (int d = 0; d < c.nd; d++)
        cd[d] = ref_dem_cell(image_pos(s.row(FD_R + d)[b] - hd * s.row(FD_VHAT0 + d)[b], sh[d], c.rmin[d], c.rmax[d]),
                             c, d);
}

/* one out-of-line copy for the count pass (out == nullptr) and the write
 * pass, so that the loop stays in the instruction cache */
__device__ __noinline__ int cpl_scan32(const DevCfg &c, const DevState &s, const int *start, int dem_base,
                                       const float4 *dpos, double hd, int64_t a, int *out, int64_t room) {
    double rad[3] = {0, 0, 0};
    float ra[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < c.nd; d++) {
        rad[d] = s.row(FD_R + d)[a];
        ra[d] = (float)rad[d];
    }
    int cs[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) cs[d] = ref_dem_cell(rad[d], c, d);
    const float lim = (float)(c.rc2 * (1.0 + 1e-4));
    float L[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < c.nd; d++) L[d] = (float)(c.rmax[d] - c.rmin[d]);
    const CellCoord cc = dem_cell_of(c, rad);
    int k = 0;
    scan_cells(cc, c.ddims, c.periodic, c.nd, start, dem_base, [&](int b, const int *sh) {
        if (s.irow(FI_IAM)[b] != T_DEM) return;
        const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
        int cd[3] = {0, 0, 0};
        if (shifted)
            image_dem_cells(c, s, b, sh, hd, cd);
        else
            for (int d = 0; d < c.nd; d++) cd[d] = s.irow(FI_RDC0 + d)[b];
        if (!coupling_rule(cs, cd, c)) return;
        const float4 p = dpos[b];
        const float pb[3] = {p.x, p.y, p.z};
        float r2 = 0.f;
        for (int d = 0; d < c.nd; d++) {
            const float dx = ra[d] - (pb[d] + (float)sh[d] * L[d]);
            r2 = fmaf(dx, dx, r2);
        }
        if (!(r2 < lim)) return;
        if ((sh[0] | sh[1] | sh[2]) && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return;
        if (out && k < room) out[k] = s.irow(FI_TAG)[b] | shift_code(sh);
        k++;
    });
    return k;
}

/* One scan per fluid particle: its partners go to a small per-thread buffer,
 * then one warp-aggregated reservation places them; a particle with more
 * partners than the buffer holds scans again straight into the table. */
constexpr int CPL_LOCAL = 16;
__global__ void k_cp_cpl_table(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n,
                               const float4 *dpos, int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = a < n && is_fluid(s.irow(FI_IAM)[a]);
    const int j = slot ? *slot : 0;
    int lb[CPL_LOCAL];
    const int k = live ? cpl_scan32(c, s, start, g->n_sph_cells, dpos, 0.5 * g->dt, a, nb ? lb : nullptr,
                                    nb ? CPL_LOCAL : 0)
                       : 0;
    const int64_t off = reserve(k, cnt + j);
    if (!nb || !live) return;
    const int64_t room = cap - off;
    int *out = nb + (int64_t)j * cap + off;
    if (k <= CPL_LOCAL) {
        if (room >= k)
            for (int q = 0; q < k; q++) out[q] = lb[q];
    } else {
        cpl_scan32(c, s, start, g->n_sph_cells, dpos, 0.5 * g->dt, a, out, room > 0 ? room : 0);
    }
    oc[(int64_t)j * n + s.irow(FI_TAG)[a]] = make_int2((int)off, room >= k ? k : 0);
}

/* FPI table, one warp per DEM particle (DEM particles follow the SPH buckets
 * in the sorted order): the lanes split the 3^d SPH-bucket stencil, the
 * exact FP64 predicate of calcFPI decides, a ballot compacts.  Each DEM
 * particle owns `per` slots of the step's table (offset w * per); more
 * partners than that mark the step overflowed (cnt > cap). */
__global__ void k_cp_fpi_table(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n, int n_dem,
                               int per, int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = start[g->n_sph_cells] + w;
    if (i >= n || s.irow(FI_IAM)[i] != T_DEM) return;
    const int j = *slot;
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[i];
    const double ha = s.row(FD_H)[i];
    const GridInfo gi = load_grid(g);
    const CellCoord cs = sph_cell_of(c, gi, ra);
    int *out = nb + (int64_t)j * cap + (int64_t)w * per;
    int k = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
            for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cs, ox, oy, oz, gi.sdims, c.periodic, c.nd, sh);
                if (lin < 0) continue;
                const int b1 = start[lin + 1];
                for (int b0 = start[lin]; b0 < b1; b0 += 32) {
                    const int b = b0 + lane;
                    bool ok = b < b1;
                    if (ok) {
                        double dx[3] = {0, 0, 0};
                        for (int d = 0; d < c.nd; d++)
                            dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
                        const double r2 = exact_len2(dx, c.nd);
                        const double hb = s.row(FD_H)[b];
                        const double t = 2.0 * (ha > hb ? ha : hb);
                        ok = r2 <= dmul(t, t) && s.irow(FI_IAM)[b] != T_BOUNDARY &&
                             (!(sh[0] | sh[1] | sh[2]) || image_exists(s.irow(FI_GCODE)[b], sh, c.nd));
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, ok);
                    const int pos = k + __popc(m & lt);
                    if (ok && pos < per) out[pos] = s.irow(FI_TAG)[b] | shift_code(sh);
                    k += __popc(m);
                }
            }
    if (lane == 0) {
        oc[(int64_t)j * n + s.irow(FI_TAG)[i]] = make_int2(w * per, k <= per ? k : 0);
        if (k > per) atomicMax(cnt + j, (int)cap + 1);   /* marks the step overflowed */
    }
}

/* contact table, one thread per DEM particle, `per` slots each */
__global__ void k_cp_ct_table(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n, int n_dem,
                              int per, int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot) {
    const int w = (int)(blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
    if (w >= n_dem) return;
    const int64_t i = start[g->n_sph_cells] + w;
    if (i >= n || s.irow(FI_IAM)[i] != T_DEM) return;
    const int j = *slot;
    int *out = nb + (int64_t)j * cap + (int64_t)w * per;
    const int k = contact_scan<true>(c, s, start, g, i, out, per);
    oc[(int64_t)j * n + s.irow(FI_TAG)[i]] = make_int2(w * per, k <= per ? k : 0);
    if (k > per) atomicMax(cnt + j, (int)cap + 1);
}

/* positions after the middle phase, tag order, at slot *slot */
__global__ void k_cp_tap_r(DevState s, int64_t n, double *rmid, const int *slot) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    double *o = rmid + ((int64_t)(*slot) * n + s.irow(FI_TAG)[k]) * 3;
    for (int d = 0; d < 3; d++) o[d] = s.row(FD_R + d)[k];
}

/* ---- reverse pass of one step ------------------------------------------ */

__device__ __forceinline__ void image_d(const DevCfg &c, const double *ra, const double *rb, const int *sh,
                                        double *d, double &r) {
    double r2 = 0.0;
    for (int q = 0; q < 3; q++) d[q] = 0.0;
    for (int q = 0; q < c.nd; q++) {
        d[q] = ra[q] - image_pos(rb[q], sh[q], c.rmin[q], c.rmax[q]);
        r2 += d[q] * d[q];
    }
    r = sqrt(r2);
}

/* coupling kernel W_c(r) = C_c K(2r/Rc) and dW_c/dr (sph.h:1246-1256) */
__device__ __forceinline__ void wc_kernel(const DevCfg &c, double r, double &W, double &Wp) {
    const double q = r * c.two_over_rc;
    W = 0.0;
    Wp = 0.0;
    if (q > 2.0) return;
    const double t = 2.0 - q, t2 = t * t;
    W = c.c_ihn * c.wcon * (t2 * t2) * (1.0 + 2.0 * q);
    Wp = c.c_ihn * c.wcon * (-10.0 * q * t2 * t) * c.two_over_rc;
}

/* intermediates: middle positions, vh_s (fluid) / vh_m (DEM), rho_s */
__global__ void k_cp_pre(int64_t n, double dt, const double *s0, const double *rm, const int *typ, double *aux) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *x = s0 + i * ADJ_NC;
    double *o = aux + i * ADJ_AUX;
    const double hd = 0.5 * dt;
    const int t = typ[i];
    for (int d = 0; d < 3; d++) {
        /* DEM: the snapshot is r_m = r_s + hd vh0 in the middle rebuild's frame */
        o[d] = t == T_DEM ? rm[i * 3 + d] - hd * x[AS_VH + d] : rm[i * 3 + d];
        o[3 + d] = (t == T_SPH || t == T_DEM) ? x[AS_VH + d] + hd * x[AS_F + d] : x[AS_VH + d];
    }
    o[6] = x[AS_DENS] + hd * x[AS_DDDT];
    o[7] = 0.0;
}

/* porosity, EOS and the Shepard sums of the middle phase (forward) */
__global__ void k_cp_por(DevCfg c, int64_t n, const double *aux, const double *mass, const int *typ, const int *nb,
                         const int2 *oc, double *cmid) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double *xa = aux + a * ADJ_AUX;
    const double rho = xa[6], dvol = mass[a] / rho;
    double e = 0.0;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int i = table_entry(nb[o.x + k], sh);
        double d[3], r, W, Wp;
        image_d(c, xa, aux + (int64_t)i * ADJ_AUX, sh, d, r);
        wc_kernel(c, r, W, Wp);
        e += c.por_incr * W;
        atomicAdd(&cmid[(int64_t)i * CP_NMID + CM_SHEP], dvol * W);
    }
    double eps = 1.0 - e;
    const bool clamp = eps < 0.37;
    if (clamp) eps = 0.37;
    const double x = rho / (c.refd * eps), x2 = x * x;
    cmid[a * CP_NMID + CM_EPS] = eps;
    cmid[a * CP_NMID + CM_CLAMP] = clamp ? 1.0 : 0.0;
    cmid[a * CP_NMID + CM_PDR2] = c.prb * (x2 * x2 * x2 * x - 1.0) / (rho * rho);
}

/* Di Felice drag Phi(dv, por) = 1/2 A C_d |dv| por^-chi dv (sph.h:1593-1598)
 * and its VJP against Pb: adds to dvb, porb, and returns the adjoint of nu */
__device__ __noinline__ void difelice(const DevCfg &c, const double *dv, double por, double *phi) {
    double vd2 = 0.0;
    for (int q = 0; q < c.nd; q++) vd2 += dv[q] * dv[q];
    const double vd = sqrt(vd2);
    for (int q = 0; q < 3; q++) phi[q] = 0.0;
    if (vd == 0.0) return;
    const double A = c.pi * c.dem_radius * c.dem_radius;
    const double Re = (2.0 * c.dem_radius / c.viscosity) * vd;
    const double lg = 1.5 - log10(Re);
    const double chi = 3.7 - 0.65 * exp(-(lg * lg) / 2.0);
    const double c0 = 0.63 + 4.8 / sqrt(Re);
    const double g = 0.5 * A * c0 * c0 * vd * pow(por, -chi);
    for (int q = 0; q < c.nd; q++) phi[q] = g * dv[q];
}

__device__ __noinline__ double difelice_vjp(const DevCfg &c, const double *dv, double por, const double *Pb,
                                               double *dvb, double &porb) {
    double vd2 = 0.0, Pd = 0.0;
    for (int q = 0; q < c.nd; q++) {
        vd2 += dv[q] * dv[q];
        Pd += Pb[q] * dv[q];
    }
    const double vd = sqrt(vd2);
    if (vd == 0.0) return 0.0;
    const double A = c.pi * c.dem_radius * c.dem_radius;
    const double Re = (2.0 * c.dem_radius / c.viscosity) * vd;
    const double lg = 1.5 - log10(Re);
    const double ex = exp(-(lg * lg) / 2.0);
    const double chi = 3.7 - 0.65 * ex;
    const double c0 = 0.63 + 4.8 / sqrt(Re);
    const double Cd = c0 * c0;
    const double g = 0.5 * A * Cd * vd;
    const double lp = log(por), Psi = exp(-chi * lp);
    const double dCd = 2.0 * c0 * (-2.4 / (Re * sqrt(Re)));         /* dC_d / dRe */
    const double dchi = -0.65 * ex * lg / (Re * log(10.0));           /* dchi / dRe */
    const double dgPsi_dRe = 0.5 * A * vd * dCd * Psi + g * (-lp * Psi * dchi);  /* at fixed |dv| */
    const double dgPsi_dvd = dgPsi_dRe * Re / vd + 0.5 * A * Cd * Psi;
    for (int q = 0; q < c.nd; q++) dvb[q] += g * Psi * Pb[q] + Pd * dgPsi_dvd * dv[q] / vd;
    porb += Pd * g * (-chi) * Psi / por;
    return Pd * dgPsi_dRe * (-Re / c.viscosity);
}

/* FPI + Di Felice drag of each DEM particle (end phase), one warp per DEM
 * particle: the lanes split its fluid partners for the forward sums (warp
 * reductions), every lane then runs the drag VJP on the reduced values, and
 * the lanes split the partners again to scatter the adjoints into the fluid
 * accumulators (FP64 atomics).  Delta_i's adjoint is that of f1 + fdrag1. */
__global__ void k_cp_fpi(DevCfg c, int n_dem, const int *dem_tags, double dt, const double *s1, const double *aux,
                         const double *cmid, const double *mass, const double *hh, const int *nb, const int2 *oc,
                         const double *adj, double *cacc, double *grads) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = dem_tags[w];
    const double *xi = s1 + i * ADJ_NC, *ai = adj + i * ADJ_NC;
    const double *vhm = aux + i * ADJ_AUX + 3;
    const int2 o = oc[i];
    double sum = 0.0, Npor = 0.0, Nfp[3] = {0, 0, 0}, Nfv[3] = {0, 0, 0}, Nvel[3] = {0, 0, 0};
    for (int k = lane; k < o.y; k += 32) {
        int sh[3];
        const int b = table_entry(nb[o.x + k], sh);
        const double *xb = s1 + (int64_t)b * ADJ_NC;
        double d[3], r;
        image_d(c, xi, xb, sh, d, r);
        const double hb = hh[b], q = r / hb;
        if (q > 2.0) continue;
        double ihn = 1.0;
        for (int dd = 0; dd < c.nd; dd++) ihn /= hb;
        const double t = 2.0 - q, t2 = t * t;
        const double W = ihn * c.wcon * (t2 * t2) * (1.0 + 2.0 * q);
        const double mb = mass[b], dvol = mb / aux[(int64_t)b * ADJ_AUX + 6];
        sum += dvol * W;
        Npor += dvol * W * cmid[(int64_t)b * CP_NMID + CM_EPS];
        for (int q3 = 0; q3 < c.nd; q3++) {
            Nfp[q3] += mb * W * xb[AS_FP + q3];
            Nfv[q3] += (mb * W + dvol * W) * xb[AS_FV + q3];
            Nvel[q3] += dvol * W * xb[AS_VH + q3];
        }
    }
    sum = warp_sum_d(sum);
    Npor = warp_sum_d(Npor);
    for (int q = 0; q < 3; q++) {
        Nfp[q] = warp_sum_d(Nfp[q]);
        Nfv[q] = warp_sum_d(Nfv[q]);
        Nvel[q] = warp_sum_d(Nvel[q]);
    }
    if (!(sum > 0.5)) return;       /* no drag, Delta = 0 (uniform over the warp) */
    const double mi = mass[i], rs = 1.0 / sum;
    const double por = Npor * rs;
    double fvel[3] = {0, 0, 0}, fpfb[3] = {0, 0, 0}, fvv[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, Db[3] = {0, 0, 0};
    for (int q = 0; q < c.nd; q++) {
        fvel[q] = Nvel[q] * rs;
        fpfb[q] = Nfp[q] * rs;
        fvv[q] = Nfv[q] * rs;
        dv[q] = por * (fvel[q] - vhm[q]);
        Db[q] = ai[AS_F + q] + dt * (ai[AS_V + q] + ai[AS_VH + q]) + ai[AS_FDRAG + q];
    }
    /* Delta = (V/m)(fv + fpfb) + (rho0/m) kappa Phi */
    double phi[3];
    difelice(c, dv, por, phi);
    double Pb[3] = {0, 0, 0}, dvb[3] = {0, 0, 0}, porb = 0.0, gkap = 0.0;
    for (int q = 0; q < c.nd; q++) {
        Pb[q] = (c.dens / mi) * c.drag_scale * Db[q];
        gkap += (c.dens / mi) * Db[q] * phi[q];
    }
    const double gnu = difelice_vjp(c, dv, por, Pb, dvb, porb);
    double fvelb[3] = {0, 0, 0}, ownvh[3] = {0, 0, 0};
    for (int q = 0; q < c.nd; q++) {
        fvelb[q] = por * dvb[q];
        ownvh[q] = -por * dvb[q];
        porb += (fvel[q] - vhm[q]) * dvb[q];
    }
    const double vm = c.dem_vol / mi;
    double sumb = -porb * por;
    double NfpB[3] = {0, 0, 0}, NfvB[3] = {0, 0, 0}, NvelB[3] = {0, 0, 0};
    for (int q = 0; q < c.nd; q++) {
        sumb -= vm * Db[q] * fpfb[q] + vm * Db[q] * fvv[q] + fvelb[q] * fvel[q];
        NfpB[q] = vm * Db[q] * rs;
        NfvB[q] = vm * Db[q] * rs;
        NvelB[q] = fvelb[q] * rs;
    }
    sumb *= rs;
    const double NporB = porb * rs;
    double own_r[3] = {0, 0, 0};
    for (int k = lane; k < o.y; k += 32) {
        int sh[3];
        const int b = table_entry(nb[o.x + k], sh);
        const double *xb = s1 + (int64_t)b * ADJ_NC;
        double d[3], r;
        image_d(c, xi, xb, sh, d, r);
        const double hb = hh[b], q = r / hb;
        if (q > 2.0) continue;
        double ihn = 1.0;
        for (int dd = 0; dd < c.nd; dd++) ihn /= hb;
        const double t = 2.0 - q, t2 = t * t;
        const double W = ihn * c.wcon * (t2 * t2) * (1.0 + 2.0 * q);
        const double Wp = ihn * c.wcon * (-10.0 * q * t2 * t) / hb;
        const double mb = mass[b], rhob = aux[(int64_t)b * ADJ_AUX + 6], dvol = mb / rhob;
        const double epsb = cmid[(int64_t)b * CP_NMID + CM_EPS];
        double vfp = 0.0, vfv = 0.0, vvel = 0.0;
        for (int q3 = 0; q3 < c.nd; q3++) {
            vfp += NfpB[q3] * xb[AS_FP + q3];
            vfv += NfvB[q3] * xb[AS_FV + q3];
            vvel += NvelB[q3] * xb[AS_VH + q3];
        }
        const double Wb = dvol * (sumb + NporB * epsb + vvel) + mb * vfp + (mb + dvol) * vfv;
        const double dvolb = W * (sumb + NporB * epsb + vvel + vfv);
        double *acc = cacc + (int64_t)b * CP_NACC;
        atomicAdd(&acc[CA_RHO], -dvolb * dvol / rhob);
        atomicAdd(&acc[CA_EPS], dvol * W * NporB);
        if (r > 0.0) {
            for (int q3 = 0; q3 < c.nd; q3++) {
                const double gq = Wb * Wp * d[q3] / r;
                own_r[q3] += gq;
                atomicAdd(&acc[CA_R1 + q3], -gq);
            }
        }
        for (int q3 = 0; q3 < c.nd; q3++) {
            atomicAdd(&acc[CA_FP + q3], mb * W * NfpB[q3]);
            atomicAdd(&acc[CA_FV + q3], (mb + dvol) * W * NfvB[q3]);
            atomicAdd(&acc[CA_VH1 + q3], dvol * W * NvelB[q3]);
        }
    }
    for (int q = 0; q < 3; q++) own_r[q] = warp_sum_d(own_r[q]);
    if (lane == 0) {
        double *acc = cacc + i * CP_NACC;
        for (int q = 0; q < c.nd; q++) {
            acc[CA_R1 + q] += own_r[q];
            acc[CA_VH1 + q] += ownvh[q];
        }
        if (gnu != 0.0 || gkap != 0.0) {
            atomicAdd(&grads[3], gnu);
            atomicAdd(&grads[4], gkap);
        }
    }
}

/* the contact term of the ordered pair (x, y) on x against the adjoint Fb of
 * f_x: adds dT/du^T Fb to ub and dT/dw^T Fb to wb (u = r_x - r_y, w = vh_x -
 * vh_y), returns the adjoints of k and gamma */
__device__ __forceinline__ void contact_vjp(const DevCfg &c, const double *u, double r, const double *w, double R2,
                                            double m, const double *Fb, double *ub, double *wb, double &gk,
                                            double &gg) {
    double nn[3] = {0, 0, 0}, wn = 0.0, Fn = 0.0;
    for (int q = 0; q < c.nd; q++) {
        nn[q] = u[q] / r;
        wn += w[q] * nn[q];
        Fn += Fb[q] * nn[q];
    }
    const double delta = R2 - r;
    const double s = c.dem_k * delta - c.dem_gamma * wn;
    for (int q = 0; q < c.nd; q++) {
        const double dsdu = -c.dem_k * nn[q] - (c.dem_gamma / r) * (w[q] - wn * nn[q]);
        ub[q] = (dsdu * Fn + (s / r) * (Fb[q] - nn[q] * Fn)) / m;
        wb[q] = -c.dem_gamma * nn[q] * Fn / m;
    }
    gk = delta * Fn / m;
    gg = -wn * Fn / m;
}

/* DEM walls and contacts at (r_m, vh_m) against F = adjoint of f1 */
__global__ void k_cp_dem(DevCfg c, int64_t n, double dt, const double *s1, const double *aux, const double *mass,
                         const double *rad, const int *typ, const int *nb, const int2 *oc, const double *adj,
                         double *cacc, double *grads) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double gk = 0.0, gg = 0.0;
    if (i < n && typ[i] == T_DEM) {
        const double *ai = adj + i * ADJ_NC, *xi = s1 + i * ADJ_NC, *vi = aux + i * ADJ_AUX + 3;
        double F[3] = {0, 0, 0}, rb[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
        for (int q = 0; q < c.nd; q++) F[q] = ai[AS_F + q] + dt * (ai[AS_V + q] + ai[AS_VH + q]);
        const double m = mass[i], R = rad[i];
        for (int w = 0; w < c.n_walls; w++) {
            double dist = 0.0, vn = 0.0, fn = 0.0;
            for (int q = 0; q < c.nd; q++) {
                dist += (xi[q] - c.wall_p[w][q]) * c.wall_n[w][q];
                vn += vi[q] * c.wall_n[w][q];
                fn += F[q] * c.wall_n[w][q];
            }
            const double overlap = R - dist;
            if (!(overlap > 0.0)) continue;
            const double qf = fn / m;
            for (int q = 0; q < c.nd; q++) {
                rb[q] += -c.dem_k * c.wall_n[w][q] * qf;
                vb[q] += -c.dem_gamma * c.wall_n[w][q] * qf;
            }
            gk += overlap * qf;
            gg += -vn * qf;
        }
        const int2 o = oc[i];
        for (int k = 0; k < o.y; k++) {
            int sh[3];
            const int j = table_entry(nb[o.x + k], sh);
            const double *xj = s1 + (int64_t)j * ADJ_NC, *vj = aux + (int64_t)j * ADJ_AUX + 3;
            const double *aj = adj + (int64_t)j * ADJ_NC;
            double u[3], r, w[3] = {0, 0, 0}, mu[3] = {0, 0, 0}, mw[3] = {0, 0, 0};
            image_d(c, xi, xj, sh, u, r);
            for (int q = 0; q < c.nd; q++) {
                w[q] = vi[q] - vj[q];
                mu[q] = -u[q];
                mw[q] = -w[q];
            }
            double ub[3], wb[3], k1, g1;
            contact_vjp(c, u, r, w, R + rad[j], m, F, ub, wb, k1, g1);
            for (int q = 0; q < c.nd; q++) {
                rb[q] += ub[q];
                vb[q] += wb[q];
            }
            gk += k1;
            gg += g1;
            /* the partner's contact (j, i): u and w flip sign */
            double Fj[3] = {0, 0, 0};
            for (int q = 0; q < c.nd; q++) Fj[q] = aj[AS_F + q] + dt * (aj[AS_V + q] + aj[AS_VH + q]);
            double k2, g2;
            contact_vjp(c, mu, r, mw, R + rad[j], mass[j], Fj, ub, wb, k2, g2);
            for (int q = 0; q < c.nd; q++) {
                rb[q] -= ub[q];
                vb[q] -= wb[q];
            }
        }
        double *acc = cacc + i * CP_NACC;
        for (int q = 0; q < c.nd; q++) {
            acc[CA_R1 + q] += rb[q];
            acc[CA_VH1 + q] += vb[q];
        }
    }
    gk = warp_sum_d(gk);
    gg = warp_sum_d(gg);
    if ((threadIdx.x & 31) == 0 && (gk != 0.0 || gg != 0.0)) {
        atomicAdd(&grads[0], gk);
        atomicAdd(&grads[1], gg);
    }
}

/* continuity (end pairs at r1), then the totals of r1, vh1 and the adjoints
 * of f1, fp, fv of each fluid particle */
__global__ void k_cp_end(DevCfg c, int64_t n, double dt, const double *s1, const double *mass, const double *hh,
                         const int *typ, const int *nb, const int2 *oc, const double *adj, const double *cacc,
                         double *cend) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double hd = 0.5 * dt;
    const double *xa = s1 + a * ADJ_NC, *aa = adj + a * ADJ_NC, *ac = cacc + a * CP_NACC;
    const double Da = aa[AS_DDDT] + hd * aa[AS_DENS], ma = mass[a], ha = hh[a];
    double rb[3] = {0, 0, 0}, wb[3] = {0, 0, 0};
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int b = table_entry(nb[o.x + k], sh);
        const double *xb = s1 + (int64_t)b * ADJ_NC, *ab = adj + (int64_t)b * ADJ_NC;
        double d[3], r, w[3] = {0, 0, 0}, wd = 0.0;
        image_d(c, xa, xb, sh, d, r);
        if (!(r > 0.0)) continue;
        for (int q = 0; q < c.nd; q++) {
            w[q] = xa[AS_VH + q] - xb[AS_VH + q];
            wd += w[q] * d[q];
        }
        double G, Gp;
        grad_factor(c, r, ha, hh[b], G, Gp);
        const double coef = mass[b] * Da + ma * (ab[AS_DDDT] + hd * ab[AS_DENS]);
        for (int q = 0; q < c.nd; q++) {
            rb[q] += coef * (G * w[q] + Gp * wd * d[q] / r);
            wb[q] += coef * G * d[q];
        }
    }
    const bool sph = typ[a] == T_SPH;
    double *ce = cend + a * CP_NEND;
    for (int q = 0; q < 3; q++) {
        const double rt = aa[AS_R + q] + ac[CA_R1 + q] + rb[q];
        const double vt = aa[AS_VH + q] + ac[CA_VH1 + q] + wb[q] + hd * rt;
        const double F = sph ? aa[AS_F + q] + dt * (vt + aa[AS_V + q]) : 0.0;
        ce[CE_R1 + q] = rt;
        ce[CE_VH1 + q] = vt;
        ce[CE_F + q] = F;
        ce[CE_P + q] = F + ac[CA_FP + q];
        ce[CE_V + q] = sph ? F + ac[CA_FV + q] : 0.0;
    }
}

/* VJP of the pressure and Morris viscous terms of the ordered pair (x, y) on
 * x: T = -m_y (pdr2_x + pdr2_y) G d + c_xy phi(r) w, against Pb (pressure
 * part) and Vb (viscous part), seen from the particle `self` (x with sign +1,
 * y with sign -1).  Adds sign * dT/dd to Db, sign * dT/dw to Wb, the adjoint
 * of rho_self (through c_xy = 2 nu rho0 m_y / (rho_x rho_y)) to Rb, of pdr2
 * (either particle's: they enter as a sum) to Qb, of nu to nub. */
__device__ __forceinline__ void cp_force_pair(const DevCfg &c, const double *d, const double *w, double r, double G,
                                              double Gp, double hbar, const double *Pb, const double *Vb, double my,
                                              double rhox, double rhoy, double pdr2x, double pdr2y, double sign,
                                              double *Db, double *Wb, double &Rb, double &Qb, double &nub) {
    const double rho_self = sign > 0.0 ? rhox : rhoy;
    double P = 0.0, Vw = 0.0;
    for (int q = 0; q < c.nd; q++) {
        P += Pb[q] * d[q];
        Vw += Vb[q] * w[q];
    }
    const double ir = 1.0 / r;
    const double s = -my * (pdr2x + pdr2y);
    Qb += -my * G * P;
    const double gpd = Gp * P * ir;
    const double eta2 = 0.01 * hbar * hbar, r2 = r * r, den = 1.0 / (r2 + eta2);
    const double phi = G * r2 * den;
    const double dphi = Gp * r2 * den + G * 2.0 * r * eta2 * den * den;
    const double cxy = 2.0 * c.viscosity * c.dens * my / (rhox * rhoy);
    const double VT = cxy * phi * Vw;
    Rb += -VT / rho_self;
    nub += VT / c.viscosity;
    for (int q = 0; q < c.nd; q++) {
        Db[q] += sign * (s * (G * Pb[q] + gpd * d[q]) + cxy * Vw * dphi * d[q] * ir);
        Wb[q] += sign * cxy * phi * Vb[q];
    }
}

/* forces of the middle phase (pairs at r_s) and the EOS: adjoints of r_s,
 * vh_s, rho_s and e of each fluid particle */
__global__ void k_cp_force(DevCfg c, int64_t n, const double *aux, const double *mass, const double *hh,
                           const int *typ, const int *nb, const int2 *oc, const double *adj, const double *cend,
                           double *cmid, double *cacc, double *grads) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double gnu = 0.0;
    if (a < n && is_fluid(typ[a])) {
        const double *xa = aux + a * ADJ_AUX, *ea = cend + a * CP_NEND;
        const double ma = mass[a], ha = hh[a], rhoa = xa[6], pa = cmid[a * CP_NMID + CM_PDR2];
        double Db[3] = {0, 0, 0}, Wb[3] = {0, 0, 0}, Rb = 0.0, Qb = 0.0, dum = 0.0;
        const int2 o = oc[a];
        for (int k = 0; k < o.y; k++) {
            int sh[3];
            const int b = table_entry(nb[o.x + k], sh);
            const double *xb = aux + (int64_t)b * ADJ_AUX, *eb = cend + (int64_t)b * CP_NEND;
            double d[3], r, w[3] = {0, 0, 0}, md[3] = {0, 0, 0}, mw[3] = {0, 0, 0};
            image_d(c, xa, xb, sh, d, r);
            if (!(r > 0.0)) continue;
            for (int q = 0; q < c.nd; q++) {
                w[q] = xa[3 + q] - xb[3 + q];
                md[q] = -d[q];
                mw[q] = -w[q];
            }
            double G, Gp;
            grad_factor(c, r, ha, hh[b], G, Gp);
            const double hbar = 0.5 * (ha + hh[b]);
            const double rhob = xb[6], pb = cmid[(int64_t)b * CP_NMID + CM_PDR2];
            cp_force_pair(c, d, w, r, G, Gp, hbar, ea + CE_P, ea + CE_V, mass[b], rhoa, rhob, pa, pb, 1.0, Db, Wb,
                          Rb, Qb, gnu);
            cp_force_pair(c, md, mw, r, G, Gp, hbar, eb + CE_P, eb + CE_V, ma, rhob, rhoa, pb, pa, -1.0, Db, Wb, Rb,
                          Qb, dum);
        }
        const double eps = cmid[a * CP_NMID + CM_EPS];
        const double x = rhoa / (c.refd * eps), x2 = x * x, x7 = x2 * x2 * x2 * x;
        const double dp_drho = c.prb * (5.0 * x7 + 2.0) / (rhoa * rhoa * rhoa);
        const double dp_deps = -7.0 * c.prb * x7 / (eps * rhoa * rhoa);
        double *ac = cacc + a * CP_NACC;
        const double *aa = adj + a * ADJ_NC;
        ac[CA_RHOS] = aa[AS_DENS] + ac[CA_RHO] + Rb + Qb * dp_drho;
        const double epsb = ac[CA_EPS] + Qb * dp_deps;
        ac[CA_EBAR] = cmid[a * CP_NMID + CM_CLAMP] != 0.0 ? 0.0 : -epsb;
        for (int q = 0; q < 3; q++) {
            ac[CA_RS + q] = ea[CE_R1 + q] + Db[q];
            cmid[a * CP_NMID + CM_VHS + q] = Wb[q];
        }
    }
    gnu = warp_sum_d(gnu);
    if ((threadIdx.x & 31) == 0 && gnu != 0.0) atomicAdd(&grads[3], gnu);
}

/* porosity and DEM -> fluid drag of the middle phase, per fluid particle */
__global__ void k_cp_cpl_a(DevCfg c, int64_t n, const double *s0, const double *aux, const double *cmid,
                           const double *cend, const double *mass, const int *typ, const int *nb, const int2 *oc,
                           double *cacc) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double *xa = aux + a * ADJ_AUX;
    double *ac = cacc + a * CP_NACC;
    const double eb = ac[CA_EBAR], rhoa = xa[6];
    const double *F = cend + a * CP_NEND + CE_F;
    const double f2d = c.nd == 2 ? 1.0 / (2.0 * c.dem_radius) : 1.0;
    double rb[3] = {0, 0, 0}, rhob = 0.0;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int i = table_entry(nb[o.x + k], sh);
        double d[3], r, W, Wp;
        image_d(c, xa, aux + (int64_t)i * ADJ_AUX, sh, d, r);
        wc_kernel(c, r, W, Wp);
        double Wbar = eb * c.por_incr;                          /* e = sum V W_c */
        const double shep = cmid[(int64_t)i * CP_NMID + CM_SHEP];
        if (shep != 0.0) {
            const double *fd0 = s0 + (int64_t)i * ADJ_NC + AS_FDRAG;
            const double mi = mass[i], sc = mi * f2d / (rhoa * shep), s = sc * W;
            double Ff = 0.0;
            double *ai = cacc + (int64_t)i * CP_NACC;
            for (int q = 0; q < c.nd; q++) {
                Ff += F[q] * fd0[q];
                atomicAdd(&ai[CA_FD0 + q], -s * F[q]);          /* fd_a = -sum s fdrag0_i */
            }
            const double sb = -Ff;
            Wbar += sb * sc;
            rhob += -sb * s / rhoa;
            atomicAdd(&ai[CA_SHEP], -sb * s / shep);
        }
        if (r > 0.0 && Wbar != 0.0) {
            double *ai = cacc + (int64_t)i * CP_NACC;
            for (int q = 0; q < c.nd; q++) {
                const double gq = Wbar * Wp * d[q] / r;
                rb[q] += gq;
                atomicAdd(&ai[CA_RS + q], -gq);
            }
        }
    }
    for (int q = 0; q < c.nd; q++) ac[CA_RS + q] += rb[q];
    ac[CA_RHOS] += rhob;
}

/* Shepard sums of the middle phase, per fluid particle */
__global__ void k_cp_cpl_b(DevCfg c, int64_t n, const double *aux, const double *mass, const int *typ,
                           const int *nb, const int2 *oc, double *cacc) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double *xa = aux + a * ADJ_AUX;
    double *ac = cacc + a * CP_NACC;
    const double rhoa = xa[6], ma = mass[a];
    double rb[3] = {0, 0, 0}, rhob = 0.0;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int i = table_entry(nb[o.x + k], sh);
        double *ai = cacc + (int64_t)i * CP_NACC;
        const double sb = ai[CA_SHEP];
        if (sb == 0.0) continue;
        double d[3], r, W, Wp;
        image_d(c, xa, aux + (int64_t)i * ADJ_AUX, sh, d, r);
        wc_kernel(c, r, W, Wp);
        rhob += -sb * ma * W / (rhoa * rhoa);
        if (r > 0.0) {
            const double Wbar = sb * ma / rhoa;
            for (int q = 0; q < c.nd; q++) {
                const double gq = Wbar * Wp * d[q] / r;
                rb[q] += gq;
                atomicAdd(&ai[CA_RS + q], -gq);
            }
        }
    }
    for (int q = 0; q < c.nd; q++) ac[CA_RS + q] += rb[q];
    ac[CA_RHOS] += rhob;
}

/* the adjoint of the state before the step */
__global__ void k_cp_assemble(int64_t n, double dt, const int *typ, const double *cacc, const double *cend,
                              const double *cmid, double *adj) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hd = 0.5 * dt;
    const int t = typ[i];
    double *aa = adj + i * ADJ_NC;
    const double *ac = cacc + i * CP_NACC;
    if (is_fluid(t)) {
        const double *ce = cend + i * CP_NEND, *cm = cmid + i * CP_NMID;
        for (int q = 0; q < 3; q++) {
            const double rs = ac[CA_RS + q], vhs = cm[CM_VHS + q];
            aa[AS_R + q] = rs;                                   /* r_s = r0 + hd vh0 */
            aa[AS_VH + q] = ce[CE_VH1 + q] + vhs + hd * rs;      /* vh1 (kick), vh_s, r_s */
            aa[AS_F + q] = t == T_SPH ? hd * vhs : 0.0;          /* vh_s = vh0 + hd f0 */
            aa[AS_FDRAG + q] = 0.0;
            aa[AS_FP + q] = 0.0;
            aa[AS_FV + q] = 0.0;
        }
        aa[AS_DENS] = ac[CA_RHOS];                               /* rho_s = rho0 + hd dddt0 */
        aa[AS_DDDT] = hd * ac[CA_RHOS];
    } else if (t == T_DEM) {
        for (int q = 0; q < 3; q++) {
            const double rmb = aa[AS_R + q] + ac[CA_R1 + q];     /* r_m */
            const double vmb = ac[CA_VH1 + q];                   /* vh_m */
            const double rsb = rmb + ac[CA_RS + q];              /* r_s = r0 + hd vh0, r_m = r_s + hd vh0 */
            aa[AS_R + q] = rsb;
            aa[AS_VH + q] = aa[AS_VH + q] + vmb + hd * rmb + hd * rsb;
            aa[AS_F + q] = hd * vmb;                             /* vh_m = vh0 + hd f0 */
            aa[AS_FDRAG + q] = ac[CA_FD0 + q];
            aa[AS_FP + q] = 0.0;
            aa[AS_FV + q] = 0.0;
        }
        aa[AS_DENS] = 0.0;
        aa[AS_DDDT] = 0.0;
    }
}

/* ---- mixed precision: FP32 pair math of the fluid pair passes ------------
 * Records per particle (float4, tag order): middle state R_M0 = (r_s hi,
 * 1/h), R_M1 = (r_s lo, m), R_M2 = (vh_s, rho_s), R_M3 = (adjoint of fp,
 * pdr2), R_M4 = (adjoint of fv, h); end state R_E0 = (r1 hi, 1/h), R_E1 =
 * (r1 lo, m), R_E2 = (vh1, adjoint of dddt1 + hd adjoint of rho1).  Pair
 * displacements come from the double-float positions; per-particle sums are
 * Kahan-compensated and land in the FP64 accumulators once. */
enum { R_M0 = 0, R_M1, R_M2, R_M3, R_M4, R_E0, R_E1, R_E2 };

__global__ void k_cp_pack32(int64_t n, double dt, const double *aux, const double *cmid, const double *s1,
                            const double *adj, const double *mass, const double *hh, const int *typ, float4 *rec) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !is_fluid(typ[i])) return;
    const double *x = aux + i * ADJ_AUX, *x1 = s1 + i * ADJ_NC, *aa = adj + i * ADJ_NC;
    const double hd = 0.5 * dt;
    const float ih = (float)(1.0 / hh[i]), m = (float)mass[i];
    float hi[3], lo[3];
    for (int d = 0; d < 3; d++) split2(x[d], hi[d], lo[d]);
    rec[R_M0 * n + i] = make_float4(hi[0], hi[1], hi[2], ih);
    rec[R_M1 * n + i] = make_float4(lo[0], lo[1], lo[2], m);
    rec[R_M2 * n + i] = make_float4((float)x[3], (float)x[4], (float)x[5], (float)x[6]);
    rec[R_M3 * n + i] = make_float4(0.f, 0.f, 0.f, (float)cmid[i * CP_NMID + CM_PDR2]);
    rec[R_M4 * n + i] = make_float4(0.f, 0.f, 0.f, (float)hh[i]);
    for (int d = 0; d < 3; d++) split2(x1[AS_R + d], hi[d], lo[d]);
    rec[R_E0 * n + i] = make_float4(hi[0], hi[1], hi[2], ih);
    rec[R_E1 * n + i] = make_float4(lo[0], lo[1], lo[2], m);
    rec[R_E2 * n + i] = make_float4((float)x1[AS_VH], (float)x1[AS_VH + 1], (float)x1[AS_VH + 2],
                                    (float)(aa[AS_DDDT] + hd * aa[AS_DENS]));
}

template <int ND>
__device__ __forceinline__ void image32(const DevCfg &c, const int *sh, float *img) {
#pragma unroll
    for (int q = 0; q < ND; q++) img[q] = sh[q] == 0 ? 0.f : (float)(sh[q] * (c.rmax[q] - c.rmin[q]));
}

/* continuity (end pairs) in FP32, then the FP64 totals of r1, vh1 and the
 * adjoints of f1, fp, fv (k_cp_end) */
template <int ND>
__global__ void __launch_bounds__(128) k_cp_end32(DevCfg c, int64_t n, double dt, const int *typ,
                                                  const int *__restrict__ nb, const int2 *__restrict__ oc,
                                                  const double *adj, const double *cacc, double *cend, float4 *rec) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const float4 *E0 = rec + R_E0 * n, *E1 = rec + R_E1 * n, *E2 = rec + R_E2 * n;
    const float wcon = (float)c.wcon;
    const float4 p0 = E0[a], p1 = E1[a], p2 = E2[a];
    const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
    Kf rb[ND], wb[ND];
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int b = table_entry(__ldg(nb + o.x + k), sh);
        float img[3];
        image32<ND>(c, sh, img);
        const float4 q0 = E0[b], q1 = E1[b], q2 = E2[b];
        const float pb[3] = {q0.x, q0.y, q0.z}, lb[3] = {q1.x, q1.y, q1.z}, vb[3] = {q2.x, q2.y, q2.z};
        float d[3], w[3], r2 = 0.f, wd = 0.f;
#pragma unroll
        for (int q = 0; q < ND; q++) {
            d[q] = ((pa[q] - pb[q]) + (la[q] - lb[q])) - img[q];
            w[q] = va[q] - vb[q];
            r2 = fmaf(d[q], d[q], r2);
            wd = fmaf(w[q], d[q], wd);
        }
        if (!(r2 > 0.f)) continue;
        const float r = sqrtf(r2);
        float G, Gp;
        grad_factor32<ND>(wcon, r, p0.w, q0.w, G, Gp);
        const float coef = q1.w * p2.w + p1.w * q2.w;
        const float gw = Gp * wd / r;
#pragma unroll
        for (int q = 0; q < ND; q++) {
            rb[q].add(coef * (G * w[q] + gw * d[q]));
            wb[q].add(coef * G * d[q]);
        }
    }
    const double hd = 0.5 * dt;
    const double *aa = adj + a * ADJ_NC, *ac = cacc + a * CP_NACC;
    const bool sph = typ[a] == T_SPH;
    double *ce = cend + a * CP_NEND;
    float P[3] = {0.f, 0.f, 0.f}, V[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < 3; q++) {
        const double rt = aa[AS_R + q] + ac[CA_R1 + q] + (q < ND ? rb[q].value() : 0.0);
        const double vt = aa[AS_VH + q] + ac[CA_VH1 + q] + (q < ND ? wb[q].value() : 0.0) + hd * rt;
        const double F = sph ? aa[AS_F + q] + dt * (vt + aa[AS_V + q]) : 0.0;
        ce[CE_R1 + q] = rt;
        ce[CE_VH1 + q] = vt;
        ce[CE_F + q] = F;
        ce[CE_P + q] = F + ac[CA_FP + q];
        ce[CE_V + q] = sph ? F + ac[CA_FV + q] : 0.0;
        P[q] = (float)ce[CE_P + q];
        V[q] = (float)ce[CE_V + q];
    }
    float4 *M3 = rec + R_M3 * n, *M4 = rec + R_M4 * n;
    M3[a] = make_float4(P[0], P[1], P[2], M3[a].w);
    M4[a] = make_float4(V[0], V[1], V[2], M4[a].w);
}

/* cp_force_pair in FP32 with Kahan sums */
template <int ND>
__device__ __forceinline__ void cp_force_pair32(float nu, float rho0, const float *d, const float *w, float r,
                                                float G, float Gp, float hbar, const float *Pb, const float *Vb,
                                                float my, float rhox, float rhoy, float pdr2x, float pdr2y,
                                                float sign, Kf *Db, Kf *Wb, Kf &Rb, Kf &Qb, float &nub) {
    float P = 0.f, Vw = 0.f;
#pragma unroll
    for (int q = 0; q < ND; q++) {
        P = fmaf(Pb[q], d[q], P);
        Vw = fmaf(Vb[q], w[q], Vw);
    }
    const float ir = 1.f / r;
    const float s = -my * (pdr2x + pdr2y);
    Qb.add(-my * G * P);
    const float gpd = Gp * P * ir;
    const float eta2 = 0.01f * hbar * hbar, r2 = r * r, den = 1.f / (r2 + eta2);
    const float phi = G * r2 * den;
    const float dphi = Gp * r2 * den + G * 2.f * r * eta2 * den * den;
    const float cxy = 2.f * nu * rho0 * my / (rhox * rhoy);
    const float VT = cxy * phi * Vw;
    Rb.add(-VT / (sign > 0.f ? rhox : rhoy));
    nub += VT / nu;
    const float cv = cxy * Vw * dphi * ir;
#pragma unroll
    for (int q = 0; q < ND; q++) {
        Db[q].add(sign * (s * (G * Pb[q] + gpd * d[q]) + cv * d[q]));
        Wb[q].add(sign * cxy * phi * Vb[q]);
    }
}

/* forces (middle pairs) in FP32 and the EOS in FP64 (k_cp_force) */
template <int ND>
__global__ void __launch_bounds__(128) k_cp_force32(DevCfg c, int64_t n, const int *typ, const int *__restrict__ nb,
                                                    const int2 *__restrict__ oc, const double *adj,
                                                    const double *aux, const double *cend,
                                                    const float4 *__restrict__ rec, double *cmid, double *cacc,
                                                    double *grads) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float gnu = 0.f;
    if (a < n && is_fluid(typ[a])) {
        const float4 *M0 = rec + R_M0 * n, *M1 = rec + R_M1 * n, *M2 = rec + R_M2 * n, *M3 = rec + R_M3 * n,
                     *M4 = rec + R_M4 * n;
        const float wcon = (float)c.wcon, nu = (float)c.viscosity, rho0 = (float)c.dens;
        const float4 p0 = M0[a], p1 = M1[a], p2 = M2[a], p3 = M3[a], p4 = M4[a];
        const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
        const float Pa[3] = {p3.x, p3.y, p3.z}, Va[3] = {p4.x, p4.y, p4.z};
        const bool own = Pa[0] != 0.f || Pa[1] != 0.f || Pa[2] != 0.f || Va[0] != 0.f || Va[1] != 0.f ||
                         Va[2] != 0.f;
        Kf Db[ND], Wb[ND], Rb, Qb;
        float dum = 0.f;
        const int2 o = oc[a];
        for (int k = 0; k < o.y; k++) {
            int sh[3];
            const int b = table_entry(__ldg(nb + o.x + k), sh);
            float img[3];
            image32<ND>(c, sh, img);
            const float4 q0 = M0[b], q1 = M1[b], q2 = M2[b], q3 = M3[b], q4 = M4[b];
            const float pb[3] = {q0.x, q0.y, q0.z}, lb[3] = {q1.x, q1.y, q1.z}, vb[3] = {q2.x, q2.y, q2.z};
            const float Pbv[3] = {q3.x, q3.y, q3.z}, Vbv[3] = {q4.x, q4.y, q4.z};
            float d[3], w[3], md[3], mw[3], r2 = 0.f;
#pragma unroll
            for (int q = 0; q < ND; q++) {
                d[q] = ((pa[q] - pb[q]) + (la[q] - lb[q])) - img[q];
                w[q] = va[q] - vb[q];
                md[q] = -d[q];
                mw[q] = -w[q];
                r2 = fmaf(d[q], d[q], r2);
            }
            if (!(r2 > 0.f)) continue;
            const float r = sqrtf(r2);
            float G, Gp;
            grad_factor32<ND>(wcon, r, p0.w, q0.w, G, Gp);
            const float hbar = 0.5f * (p4.w + q4.w);
            if (own)
                cp_force_pair32<ND>(nu, rho0, d, w, r, G, Gp, hbar, Pa, Va, q1.w, p2.w, q2.w, p3.w, q3.w, 1.f, Db, Wb,
                                    Rb, Qb, gnu);
            if (Pbv[0] != 0.f || Pbv[1] != 0.f || Pbv[2] != 0.f || Vbv[0] != 0.f || Vbv[1] != 0.f || Vbv[2] != 0.f)
                cp_force_pair32<ND>(nu, rho0, md, mw, r, G, Gp, hbar, Pbv, Vbv, p1.w, q2.w, p2.w, q3.w, p3.w, -1.f, Db,
                                    Wb, Rb, Qb, dum);
        }
        const double rhoa = aux[a * ADJ_AUX + 6];
        const double eps = cmid[a * CP_NMID + CM_EPS];
        const double x = rhoa / (c.refd * eps), x2 = x * x, x7 = x2 * x2 * x2 * x;
        const double dp_drho = c.prb * (5.0 * x7 + 2.0) / (rhoa * rhoa * rhoa);
        const double dp_deps = -7.0 * c.prb * x7 / (eps * rhoa * rhoa);
        double *ac = cacc + a * CP_NACC;
        const double *aa = adj + a * ADJ_NC, *ea = cend + a * CP_NEND;
        const double Qv = Qb.value();
        ac[CA_RHOS] = aa[AS_DENS] + ac[CA_RHO] + Rb.value() + Qv * dp_drho;
        const double epsb = ac[CA_EPS] + Qv * dp_deps;
        ac[CA_EBAR] = cmid[a * CP_NMID + CM_CLAMP] != 0.0 ? 0.0 : -epsb;
        for (int q = 0; q < 3; q++) {
            ac[CA_RS + q] = ea[CE_R1 + q] + (q < ND ? Db[q].value() : 0.0);
            cmid[a * CP_NMID + CM_VHS + q] = q < ND ? Wb[q].value() : 0.0;
        }
    }
    gnu += __shfl_xor_sync(0xffffffffu, gnu, 16);
    gnu += __shfl_xor_sync(0xffffffffu, gnu, 8);
    gnu += __shfl_xor_sync(0xffffffffu, gnu, 4);
    gnu += __shfl_xor_sync(0xffffffffu, gnu, 2);
    gnu += __shfl_xor_sync(0xffffffffu, gnu, 1);
    if ((threadIdx.x & 31) == 0 && gnu != 0.f) atomicAdd(&grads[3], (double)gnu);
}

}  // namespace

void cpl_count_tables(sphdem_ctx *c, AdjointData *a) {
    /* the coupling pairs of the current buckets, counted with the tap's own
     * scan (a->slot is a device int the replay resets before use) */
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->dpos, (size_t)c->n * sizeof(float4)));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->slot, 0, sizeof(int), c->stream));
    k_cp_dpos<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->g, c->n, a->dpos);
    k_cp_cpl_table<<<grid_for(c->n, CB), CB, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, c->n, a->dpos,
                                                             nullptr, nullptr, a->slot, 0, nullptr);
    int nc = 0;
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(&nc, a->slot, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    a->cpl.cap = (int64_t)nc + nc / 2 + 4096;
    std::vector<int> iam(c->n), tags;
    field_get_int(c, FI_IAM, iam.data());   /* tag order */
    for (int64_t i = 0; i < c->n; i++)
        if (iam[i] == T_DEM) tags.push_back((int)i);
    a->n_dem = (int)tags.size();
    a->fpi.cap = (int64_t)std::max(1, a->n_dem) * CP_FPI_PER;
    a->ct_cap = (int64_t)std::max(1, a->n_dem) * ADJ_MAX_CONTACTS;
    if (!tags.empty()) {
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->dem_tags, tags.size() * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMemcpy(a->dem_tags, tags.data(), tags.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
}

void cpl_alloc(sphdem_ctx *c, AdjointData *a) {
    const int K = a->K;
    const int64_t n = c->n;
    a->cpl.alloc(K, n);
    a->fpi.alloc(K, n);
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.nb, (size_t)K * a->ct_cap * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.oc, (size_t)K * n * sizeof(int2)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.cnt, (size_t)K * sizeof(int)));
    a->ct.cap = a->ct_cap;
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->rmid, (size_t)K * n * 3 * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->cacc, (size_t)n * CP_NACC * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->cend, (size_t)n * CP_NEND * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->cmid, (size_t)n * CP_NMID * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->aux, (size_t)n * ADJ_AUX * sizeof(double)));
    if (c->cfg.precision == SPHDEM_PREC_MIXED)
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->crec, (size_t)n * CP_NREC32 * sizeof(float4)));
}

void cpl_free(AdjointData *a) {
    a->cpl.free_all();
    a->fpi.free_all();
    a->ct.free_all();
    cudaFree(a->rmid);
    cudaFree(a->cacc);
    cudaFree(a->cend);
    cudaFree(a->cmid);
    cudaFree(a->crec);
    cudaFree(a->dpos);
    cudaFree(a->dem_tags);
    a->rmid = a->cacc = a->cend = a->cmid = nullptr;
    a->crec = nullptr;
    a->dpos = nullptr;
    a->dem_tags = nullptr;
}

void cpl_reset_segment(sphdem_ctx *c, AdjointData *a) {
    const size_t ocb = (size_t)a->K * c->n * sizeof(int2);
    for (PairTable *t : {&a->cpl, &a->fpi, &a->ct}) {
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(t->oc, 0, ocb, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(t->cnt, 0, a->K * sizeof(int), c->stream));
    }
}

void cpl_taps_middle(sphdem_ctx *c, AdjointData *a) {
    k_cp_dpos<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->g, c->n, a->dpos);
    k_cp_cpl_table<<<grid_for(c->n, CB), CB, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, c->n, a->dpos,
                                                             a->cpl.nb, a->cpl.oc, a->cpl.cnt, a->cpl.cap, a->slot);
    k_cp_tap_r<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->n, a->rmid, a->slot);
}

void cpl_taps_end(sphdem_ctx *c, AdjointData *a) {
    if (a->n_dem == 0) return;
    k_cp_fpi_table<<<grid_for((int64_t)a->n_dem * 32, CB), CB, 0, c->stream>>>(
        c->cfg, c->A, c->buf.start, c->g, c->n, a->n_dem, CP_FPI_PER, a->fpi.nb, a->fpi.oc, a->fpi.cnt, a->fpi.cap,
        a->slot);
    k_cp_ct_table<<<grid_for(a->n_dem, CB), CB, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, c->n, a->n_dem,
                                                                ADJ_MAX_CONTACTS, a->ct.nb, a->ct.oc, a->ct.cnt,
                                                                a->ct.cap, a->slot);
}

bool cpl_overflow(sphdem_ctx *c, AdjointData *a) {
    std::vector<int> v(3 * a->K);
    const PairTable *ts[3] = {&a->cpl, &a->fpi, &a->ct};
    for (int k = 0; k < 3; k++)
        SPHDEM_CUDA_CHECK(
            cudaMemcpyAsync(v.data() + k * a->K, ts[k]->cnt, a->K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 3; k++)
        for (int j = 0; j < a->K; j++)
            if (v[k * a->K + j] > ts[k]->cap) return true;
    return false;
}

void cpl_backward_step(sphdem_ctx *c, AdjointData *a, int j, double dt) {
    const int64_t n = c->n;
    const double *s0 = a->seg + (size_t)(j - 1) * n * ADJ_NC, *s1 = a->seg + (size_t)j * n * ADJ_NC;
    const double *rm = a->rmid + (size_t)(j - 1) * n * 3;
    const int sl = j - 1;
    auto nbp = [&](const PairTable &t) { return t.nb + (size_t)sl * t.cap; };
    auto ocp = [&](const PairTable &t) { return t.oc + (size_t)sl * n; };
    const int *nbm = a->nb_mid + (size_t)sl * a->pair_cap, *nbe = a->nb_end + (size_t)sl * a->pair_cap;
    const int2 *ocm = a->oc_mid + (size_t)sl * n, *oce = a->oc_end + (size_t)sl * n;
    const int g = grid_for(n, CB);
    cudaStream_t st = c->stream;
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->cacc, 0, (size_t)n * CP_NACC * sizeof(double), st));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->cmid, 0, (size_t)n * CP_NMID * sizeof(double), st));
    k_cp_pre<<<grid_for(n, 256), 256, 0, st>>>(n, dt, s0, rm, a->typ, a->aux);
    k_cp_por<<<g, CB, 0, st>>>(c->cfg, n, a->aux, a->mass, a->typ, nbp(a->cpl), ocp(a->cpl), a->cmid);
    if (a->n_dem > 0)
        k_cp_fpi<<<grid_for((int64_t)a->n_dem * 32, CB), CB, 0, st>>>(c->cfg, a->n_dem, a->dem_tags, dt, s1, a->aux,
                                                                      a->cmid, a->mass, a->hh, nbp(a->fpi),
                                                                      ocp(a->fpi), a->adj, a->cacc, a->grads);
    k_cp_dem<<<g, CB, 0, st>>>(c->cfg, n, dt, s1, a->aux, a->mass, a->rad, a->typ, nbp(a->ct), ocp(a->ct), a->adj,
                               a->cacc, a->grads);
    if (a->crec) {
        k_cp_pack32<<<grid_for(n, 256), 256, 0, st>>>(n, dt, a->aux, a->cmid, s1, a->adj, a->mass, a->hh, a->typ,
                                                       a->crec);
#define L_(ND)                                                                                                   \
    do {                                                                                                         \
        k_cp_end32<ND><<<g, CB, 0, st>>>(c->cfg, n, dt, a->typ, nbe, oce, a->adj, a->cacc, a->cend, a->crec);     \
        k_cp_force32<ND><<<g, CB, 0, st>>>(c->cfg, n, a->typ, nbm, ocm, a->adj, a->aux, a->cend, a->crec, a->cmid, \
                                           a->cacc, a->grads);                                                    \
    } while (0)
        if (c->cfg.nd == 3) L_(3);
        else if (c->cfg.nd == 2) L_(2);
        else L_(1);
#undef L_
    } else {
        k_cp_end<<<g, CB, 0, st>>>(c->cfg, n, dt, s1, a->mass, a->hh, a->typ, nbe, oce, a->adj, a->cacc, a->cend);
        k_cp_force<<<g, CB, 0, st>>>(c->cfg, n, a->aux, a->mass, a->hh, a->typ, nbm, ocm, a->adj, a->cend, a->cmid,
                                     a->cacc, a->grads);
    }
    k_cp_cpl_a<<<g, CB, 0, st>>>(c->cfg, n, s0, a->aux, a->cmid, a->cend, a->mass, a->typ, nbp(a->cpl), ocp(a->cpl),
                                 a->cacc);
    k_cp_cpl_b<<<g, CB, 0, st>>>(c->cfg, n, a->aux, a->mass, a->typ, nbp(a->cpl), ocp(a->cpl), a->cacc);
    k_cp_assemble<<<grid_for(n, 256), 256, 0, st>>>(n, dt, a->typ, a->cacc, a->cend, a->cmid, a->adj);
}

}  // namespace sphdem
