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
 * step runs, in order: the transposed coupling and FPI tables of the step
 * (transpose), intermediates (k_cp_pre), porosity / EOS (k_cp_por), Shepard
 * sums (k_cp_shep), FPI + drag (k_cp_fpi on the DEM side, k_cp_fpi_fluid on
 * the fluid side), DEM walls + contacts (k_cp_dem), continuity and the
 * adjoint of f1 (k_cp_end), forces + EOS (k_cp_force), porosity, DEM->fluid
 * drag and Shepard terms (k_cp_cpl_dem, k_cp_cpl_fluid) and the adjoint of
 * the state before the step (k_cp_assemble).  Every pair term is gathered by
 * both of its particles (the fluid over the symmetric pair tables, fluid <->
 * DEM over a table and its transpose), so no accumulator takes an atomic;
 * only the five scalar gradients are reduced with one FP64 atomic per warp.
 *
 * Mixed-precision handles take the coupling, FPI and contact tables from
 * the forward passes themselves (k_couple, k_dem_end write them while the
 * replay graph runs); FP64 handles scan for them after each phase.
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
#include <cstdlib>
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
    CA_EBAR = 22,   /* fluid: adjoint of e = 1 - eps (0 where clamped) */
    CA_HB = 23      /* fluid, VAR_H_CORRECTION: adjoint of h_s */
};
/* end-phase results (CP_NEND): total adjoint of r1, vh1, f1, fp, fv */
enum : int { CE_R1 = 0, CE_VH1 = 3, CE_F = 6, CE_P = 9, CE_V = 12 };
/* middle intermediates (CP_NMID): eps, clamped, pdr2, Shepard sum (DEM),
 * adjoint of vh_s, 1 / Shepard sum (DEM; 0 for a zero sum) */
enum : int { CM_EPS = 0, CM_CLAMP = 1, CM_PDR2 = 2, CM_SHEP = 3, CM_VHS = 4, CM_ISHEP = 7 };
/* FPI coefficient record of a DEM particle (CP_NCOEF): drag on (1) or not
 * (0), then the adjoints of its Shepard sum, of the porosity sum and of the
 * fp, fv and velocity sums */
enum : int { CF_ON = 0, CF_SUM = 1, CF_POR = 2, CF_FP = 3, CF_FV = 6, CF_VEL = 9 };

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

/* positions and Omega of the force pass after the middle phase, tag order,
 * at slot *slot */
__global__ void k_cp_tap_r(DevState s, int64_t n, double *rmid, const int *slot) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    double *o = rmid + ((int64_t)(*slot) * n + s.irow(FI_TAG)[k]) * RM_NC;
    for (int d = 0; d < 3; d++) o[d] = s.row(FD_R + d)[k];
    o[3] = s.row(FD_OMEGA)[k];
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

/* intermediates: middle positions, vh_s (fluid) / vh_m (DEM), rho_s, 1/rho_s;
 * with hs (VAR_H_CORRECTION): the step's smoothing length h_s = hfac (m /
 * rho_s)^(1/d) of the fluid (the start phase's update), hh of the rest */
__global__ void k_cp_pre(int64_t n, double dt, const double *s0, const double *rm, const int *typ, double *aux,
                         const double *mass, const double *hh, double *hs, double hfac, int nd) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *x = s0 + i * ADJ_NC;
    double *o = aux + i * ADJ_AUX;
    const double hd = 0.5 * dt;
    const int t = typ[i];
    for (int d = 0; d < 3; d++) {
        /* DEM: the snapshot is r_m = r_s + hd vh0 in the middle rebuild's frame */
        o[d] = t == T_DEM ? rm[i * RM_NC + d] - hd * x[AS_VH + d] : rm[i * RM_NC + d];
        o[3 + d] = (t == T_SPH || t == T_DEM) ? x[AS_VH + d] + hd * x[AS_F + d] : x[AS_VH + d];
    }
    o[6] = x[AS_DENS] + hd * x[AS_DDDT];
    o[7] = is_fluid(t) ? 1.0 / o[6] : 0.0;
    if (hs) hs[i] = is_fluid(t) ? hfac * pow(mass[i] * o[7], 1.0 / nd) : hh[i];
}

/* ---- pair geometry of the coupling and FPI tables -------------------------
 * Each coupling pair is visited by four reverse passes and each FPI pair by
 * three; its displacement, kernel value and kernel slope are evaluated once
 * per step into records of the pair's table entry: g4 = (d, W'/r), gw = W.
 * M = float on mixed-precision handles (the displacement is an FP64
 * difference rounded once), double on FP64 handles. */
template <typename M> struct MT;
template <> struct MT<float> {
    using V4 = float4;
    using Acc = Kf;
    static __device__ __forceinline__ float4 make(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
    static __device__ __forceinline__ float root(float x) { return sqrtf(x); }
};
/* plain FP64 sum with Kf's interface */
struct Kd {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct MT<double> {
    using V4 = double4;
    using Acc = Kd;
    static __device__ __forceinline__ double4 make(double a, double b, double c, double d) {
        return make_double4(a, b, c, d);
    }
    static __device__ __forceinline__ double root(double x) { return sqrt(x); }
};

/* dW/dh(r, h) = -C h^-(d+1) (d K(q) + q K'(q)) */
template <int ND, typename M>
__device__ __forceinline__ M w_dh(M wcon, M r, M ih) {
    const M q = r * ih;
    if (q > (M)2) return (M)0;
    const M t = (M)2 - q, t2 = t * t;
    M ihd1 = ih;
#pragma unroll
    for (int d = 0; d < ND; d++) ihd1 *= ih;
    return -wcon * ihd1 * (t2 * t * ((M)ND * t * ((M)1 + (M)2 * q) - (M)10 * q * q));
}

/* coupling pairs, one thread per fluid particle: d = r_a - r_i at the middle
 * positions, W = W_c(r) = C_c K(2r/Rc) and W_c'(r) / r (sph.h:1246-1256) */
template <typename M>
__global__ void k_cp_geo_cpl(DevCfg c, int64_t n, const double *aux, const int *typ, const int *nb, const int2 *oc,
                             typename MT<M>::V4 *g4, M *gw) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double *xa = aux + a * ADJ_AUX;
    const M tor = (M)c.two_over_rc, cw = (M)(c.c_ihn * c.wcon);
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        const int e = o.x + k;
        int sh[3];
        const int i = table_entry(nb[e], sh);
        M d[3] = {0, 0, 0}, r2 = 0;
        for (int q = 0; q < c.nd; q++) {
            d[q] = (M)(xa[q] - image_pos(aux[(int64_t)i * ADJ_AUX + q], sh[q], c.rmin[q], c.rmax[q]));
            r2 += d[q] * d[q];
        }
        const M r = MT<M>::root(r2), qq = r * tor;
        M W = 0, wpr = 0;
        if (!(qq > (M)2)) {
            const M t = (M)2 - qq, t2 = t * t;
            W = cw * (t2 * t2) * ((M)1 + (M)2 * qq);
            if (r > (M)0) wpr = cw * ((M)-10 * qq * t2 * t) * tor / r;
        }
        g4[e] = MT<M>::make(d[0], d[1], d[2], wpr);
        gw[e] = W;
    }
}

/* FPI pairs, one warp per DEM particle: d = r_i - r_b at the end positions,
 * W = W(r / h_b, h_b) and W' / r with the fluid particle's h (sph.h:1708-1792) */
template <typename M>
__global__ void k_cp_geo_fpi(DevCfg c, int n_dem, const int *dem_tags, const double *s1, const double *hh,
                             const int *nb, const int2 *oc, typename MT<M>::V4 *g4, M *gw) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = dem_tags[w];
    const double *xi = s1 + i * ADJ_NC;
    const M wcon = (M)c.wcon;
    const int2 o = oc[i];
    for (int k = lane; k < o.y; k += 32) {
        const int e = o.x + k;
        int sh[3];
        const int b = table_entry(nb[e], sh);
        M d[3] = {0, 0, 0}, r2 = 0;
        for (int q = 0; q < c.nd; q++) {
            d[q] = (M)(xi[q] - image_pos(s1[(int64_t)b * ADJ_NC + q], sh[q], c.rmin[q], c.rmax[q]));
            r2 += d[q] * d[q];
        }
        const M r = MT<M>::root(r2), ih = (M)1 / (M)hh[b], qq = r * ih;
        M W = 0, wpr = 0;
        if (!(qq > (M)2)) {
            M ihn = 1;
            for (int dd = 0; dd < c.nd; dd++) ihn *= ih;
            const M t = (M)2 - qq, t2 = t * t;
            W = ihn * wcon * (t2 * t2) * ((M)1 + (M)2 * qq);
            if (r > (M)0) wpr = ihn * wcon * ((M)-10 * qq * t2 * t) * ih / r;
        }
        g4[e] = MT<M>::make(d[0], d[1], d[2], wpr);
        gw[e] = W;
    }
}

/* porosity and EOS of the middle phase (forward), per fluid particle */
template <typename M>
__global__ void k_cp_por(DevCfg c, int64_t n, const double *aux, const int *typ, const int2 *oc, const M *gw,
                         double *cmid) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const double rho = aux[a * ADJ_AUX + 6];
    typename MT<M>::Acc sw;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) sw.add(gw[o.x + k]);
    const double e = c.por_incr * sw.value();
    double eps = 1.0 - e;
    const bool clamp = eps < 0.37;
    if (clamp) eps = 0.37;
    const double x = rho / (c.refd * eps), x2 = x * x;
    cmid[a * CP_NMID + CM_EPS] = eps;
    cmid[a * CP_NMID + CM_CLAMP] = clamp ? 1.0 : 0.0;
    cmid[a * CP_NMID + CM_PDR2] = c.prb * (x2 * x2 * x2 * x - 1.0) / (rho * rho);
}

/* Shepard sums of the middle phase (forward, calcShepSum sph.h:1303-1320),
 * one warp per DEM particle over its fluid partners (transposed coupling
 * table): shep_i = sum_a (m_a / rho_a) W_c(r_ai); also 1 / shep_i */
template <typename M>
__global__ void k_cp_shep(int n_dem, const int *dem_tags, const double *aux, const double *mass, const int *nbT,
                          const int *ixT, const int2 *ocT, const M *gw, double *cmid) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = dem_tags[w];
    const int2 o = ocT[i];
    typename MT<M>::Acc s;
    for (int k = lane; k < o.y; k += 32) {
        const int a = nbT[o.x + k] & ((1 << SH_SHIFT) - 1);
        s.add((M)(mass[a] * aux[(int64_t)a * ADJ_AUX + 7]) * gw[ixT[o.x + k]]);
    }
    const double sum = warp_sum_d(s.value());
    if (lane == 0) {
        cmid[i * CP_NMID + CM_SHEP] = sum;
        cmid[i * CP_NMID + CM_ISHEP] = sum != 0.0 ? 1.0 / sum : 0.0;
    }
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
 * reductions), every lane then runs the drag VJP on the reduced values and
 * the lanes split the partners again for the particle's own position
 * adjoint.  The adjoints of the normalised sums go to the particle's
 * coefficient record (CF_*), from which k_cp_fpi_fluid gathers each fluid
 * particle's share.  Delta_i's adjoint is that of f1 + fdrag1.  Pair math in
 * M, per-particle math in FP64. */
template <typename M>
__global__ void k_cp_fpi(DevCfg c, int n_dem, const int *dem_tags, double dt, const double *s1, const double *aux,
                         const double *cmid, const double *mass, const int *nb, const int2 *oc,
                         const typename MT<M>::V4 *g4, const M *gw, const double *adj, double *cacc, double *coef,
                         double *grads) {
    using Acc = typename MT<M>::Acc;
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = dem_tags[w];
    const double *ai = adj + i * ADJ_NC;
    const double *vhm = aux + i * ADJ_AUX + 3;
    double *cf = coef + i * CP_NCOEF;
    const int2 o = oc[i];
    Acc sum, Npor, Nfp[3], Nfv[3], Nvel[3];
    for (int k = lane; k < o.y; k += 32) {
        const M W = gw[o.x + k];
        if (W == (M)0) continue;
        const int b = nb[o.x + k] & ((1 << SH_SHIFT) - 1);
        const double *xb = s1 + (int64_t)b * ADJ_NC;
        const M mb = (M)mass[b], dW = (M)(mass[b] * aux[(int64_t)b * ADJ_AUX + 7]) * W, mW = mb * W;
        sum.add(dW);
        Npor.add(dW * (M)cmid[(int64_t)b * CP_NMID + CM_EPS]);
        for (int q3 = 0; q3 < c.nd; q3++) {
            Nfp[q3].add(mW * (M)xb[AS_FP + q3]);
            Nfv[q3].add((mW + dW) * (M)xb[AS_FV + q3]);
            Nvel[q3].add(dW * (M)xb[AS_VH + q3]);
        }
    }
    const double sumv = warp_sum_d(sum.value());
    if (!(sumv > 0.5)) {             /* no drag, Delta = 0 (uniform over the warp) */
        if (lane == 0) cf[CF_ON] = 0.0;
        return;
    }
    double npor = warp_sum_d(Npor.value()), nfp[3], nfv[3], nvel[3];
    for (int q = 0; q < 3; q++) {
        nfp[q] = warp_sum_d(Nfp[q].value());
        nfv[q] = warp_sum_d(Nfv[q].value());
        nvel[q] = warp_sum_d(Nvel[q].value());
    }
    /* the particle's own FP64 math (drag law and its VJP, with its
     * transcendentals) once per warp, on lane 0; the lanes take the adjoints
     * of the sums from its coefficient record */
    if (lane == 0) {
        const double mi = mass[i], rs = 1.0 / sumv;
        const double por = npor * rs;
        double fvel[3] = {0, 0, 0}, fpfb[3] = {0, 0, 0}, fvv[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, Db[3] = {0, 0, 0};
        for (int q = 0; q < c.nd; q++) {
            fvel[q] = nvel[q] * rs;
            fpfb[q] = nfp[q] * rs;
            fvv[q] = nfv[q] * rs;
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
        double fvelb[3] = {0, 0, 0};
        double *acc = cacc + i * CP_NACC;
        for (int q = 0; q < c.nd; q++) {
            fvelb[q] = por * dvb[q];
            acc[CA_VH1 + q] += -por * dvb[q];
            porb += (fvel[q] - vhm[q]) * dvb[q];
        }
        const double vm = c.dem_vol / mi;
        double sumb = -porb * por;
        cf[CF_ON] = 1.0;
        for (int q = 0; q < 3; q++) {
            const bool on = q < c.nd;
            if (on) sumb -= vm * Db[q] * fpfb[q] + vm * Db[q] * fvv[q] + fvelb[q] * fvel[q];
            cf[CF_FP + q] = on ? vm * Db[q] * rs : 0.0;
            cf[CF_FV + q] = on ? vm * Db[q] * rs : 0.0;
            cf[CF_VEL + q] = on ? fvelb[q] * rs : 0.0;
        }
        cf[CF_SUM] = sumb * rs;
        cf[CF_POR] = porb * rs;
        if (gnu != 0.0 || gkap != 0.0) {
            atomicAdd(&grads[3], gnu);
            atomicAdd(&grads[4], gkap);
        }
    }
    __syncwarp();
    const M sumbM = (M)cf[CF_SUM], NporBM = (M)cf[CF_POR];
    M NfpBM[3], NfvBM[3], NvelBM[3];
    for (int q = 0; q < 3; q++) {
        NfpBM[q] = (M)cf[CF_FP + q];
        NfvBM[q] = (M)cf[CF_FV + q];
        NvelBM[q] = (M)cf[CF_VEL + q];
    }
    Acc own_r[3];
    for (int k = lane; k < o.y; k += 32) {
        const typename MT<M>::V4 gd = g4[o.x + k];
        if (gd.w == (M)0) continue;
        const int b = nb[o.x + k] & ((1 << SH_SHIFT) - 1);
        const double *xb = s1 + (int64_t)b * ADJ_NC;
        const M mb = (M)mass[b], dvol = (M)(mass[b] * aux[(int64_t)b * ADJ_AUX + 7]);
        const M epsb = (M)cmid[(int64_t)b * CP_NMID + CM_EPS];
        M vfp = 0, vfv = 0, vvel = 0;
        for (int q3 = 0; q3 < c.nd; q3++) {
            vfp += NfpBM[q3] * (M)xb[AS_FP + q3];
            vfv += NfvBM[q3] * (M)xb[AS_FV + q3];
            vvel += NvelBM[q3] * (M)xb[AS_VH + q3];
        }
        const M Wb = dvol * (sumbM + NporBM * epsb + vvel) + mb * vfp + (mb + dvol) * vfv;
        const M dd[3] = {gd.x, gd.y, gd.z};
        for (int q3 = 0; q3 < c.nd; q3++) own_r[q3].add(Wb * gd.w * dd[q3]);
    }
    double own[3];
    for (int q = 0; q < 3; q++) own[q] = warp_sum_d(own_r[q].value());
    if (lane == 0) {
        double *acc = cacc + i * CP_NACC;
        for (int q = 0; q < c.nd; q++) acc[CA_R1 + q] += own[q];
    }
}

/* the fluid side of k_cp_fpi: each fluid particle gathers, over its DEM FPI
 * partners (transposed FPI table), the adjoints of its density, porosity,
 * end position, velocity and force parts that the partners' normalised sums
 * give it */
template <typename M, bool VH>
__global__ void k_cp_fpi_fluid(int64_t n, int nd, const double *s1, const double *aux, const double *cmid,
                               const double *mass, const int *typ, const int *nbT, const int *ixT, const int2 *ocT,
                               const typename MT<M>::V4 *g4, const M *gw, const double *coef, double *cacc,
                               const double *hp, double wcon) {
    using Acc = typename MT<M>::Acc;
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= n || !is_fluid(typ[b])) return;
    const int2 o = ocT[b];
    if (o.y == 0) return;
    const double *xb = s1 + b * ADJ_NC;
    const M mb = (M)mass[b], irho = (M)aux[b * ADJ_AUX + 7], dvol = (M)(mass[b] * aux[b * ADJ_AUX + 7]);
    const M epsb = (M)cmid[b * CP_NMID + CM_EPS];
    M fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, vh[3] = {0, 0, 0};
    for (int q = 0; q < nd; q++) {
        fp[q] = (M)xb[AS_FP + q];
        fv[q] = (M)xb[AS_FV + q];
        vh[q] = (M)xb[AS_VH + q];
    }
    Acc arho, aeps, ar[3], afp[3], afv[3], avh[3], ahs;
    const M ihb = VH ? (M)(1.0 / hp[b]) : (M)0, wc = (M)wcon;
    for (int k = 0; k < o.y; k++) {
        const int e = ixT[o.x + k];
        const M W = gw[e];
        if (W == (M)0) continue;
        const int i = nbT[o.x + k] & ((1 << SH_SHIFT) - 1);
        const double *cf = coef + (int64_t)i * CP_NCOEF;
        if (cf[CF_ON] == 0.0) continue;
        const typename MT<M>::V4 gd = g4[e];                   /* d = r_i - r_b */
        const M sumb = (M)cf[CF_SUM], NporB = (M)cf[CF_POR];
        M cfp[3], cfv[3], cvel[3], vfp = 0, vfv = 0, vvel = 0;
        for (int q3 = 0; q3 < 3; q3++) {
            cfp[q3] = (M)cf[CF_FP + q3];
            cfv[q3] = (M)cf[CF_FV + q3];
            cvel[q3] = (M)cf[CF_VEL + q3];
            vfp += cfp[q3] * fp[q3];
            vfv += cfv[q3] * fv[q3];
            vvel += cvel[q3] * vh[q3];
        }
        const M Wb = dvol * (sumb + NporB * epsb + vvel) + mb * vfp + (mb + dvol) * vfv;
        const M dvolb = W * (sumb + NporB * epsb + vvel + vfv);
        arho.add(-dvolb * dvol * irho);
        aeps.add(dvol * W * NporB);
        const M dd[3] = {gd.x, gd.y, gd.z};
        if (VH) {
            /* VAR_H_CORRECTION: W(r / h_b, h_b) follows the fluid particle's h */
            const M r = MT<M>::root(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
            M wdh = 0;
            if (nd == 3) wdh = w_dh<3, M>(wc, r, ihb);
            else if (nd == 2) wdh = w_dh<2, M>(wc, r, ihb);
            else wdh = w_dh<1, M>(wc, r, ihb);
            ahs.add(Wb * wdh);
        }
        for (int q3 = 0; q3 < nd; q3++) {
            ar[q3].add(-Wb * gd.w * dd[q3]);
            afp[q3].add(mb * W * cfp[q3]);
            afv[q3].add((mb + dvol) * W * cfv[q3]);
            avh[q3].add(dvol * W * cvel[q3]);
        }
    }
    double *acc = cacc + b * CP_NACC;
    acc[CA_RHO] += arho.value();
    acc[CA_EPS] += aeps.value();
    if (VH) acc[CA_HB] += ahs.value();
    for (int q = 0; q < nd; q++) {
        acc[CA_R1 + q] += ar[q].value();
        acc[CA_FP + q] += afp[q].value();
        acc[CA_FV + q] += afv[q].value();
        acc[CA_VH1 + q] += avh[q].value();
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

/* Porosity (e = sum V W_c), DEM -> fluid drag and Shepard sums of the middle
 * phase, DEM side: one warp per DEM particle over its fluid partners
 * (transposed coupling table).  The particle's adjoints of the lagged drag
 * fdrag0 and of its Shepard sum come first (warp sums), then its position
 * adjoint from both the drag / porosity terms and the Shepard terms. */
template <typename M>
__global__ void k_cp_cpl_dem(DevCfg c, int n_dem, const int *dem_tags, const double *s0, const double *aux,
                             const double *cmid, const double *cend, const double *mass, const int *nbT,
                             const int *ixT, const int2 *ocT, const typename MT<M>::V4 *g4, const M *gw,
                             double *cacc) {
    using Acc = typename MT<M>::Acc;
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t i = dem_tags[w];
    const int2 o = ocT[i];
    const double f2d = c.nd == 2 ? 1.0 / (2.0 * c.dem_radius) : 1.0;
    const double shep = cmid[i * CP_NMID + CM_SHEP], ishep = cmid[i * CP_NMID + CM_ISHEP];
    const M Ki = (M)(mass[i] * f2d * ishep), ishepM = (M)ishep, pinc = (M)c.por_incr;
    M fd0[3] = {0, 0, 0};
    for (int q = 0; q < c.nd; q++) fd0[q] = (M)s0[i * ADJ_NC + AS_FDRAG + q];
    Acc fd0b[3], shepb, rs[3];
    for (int k = lane; k < o.y; k += 32) {
        const int e = ixT[o.x + k], a = nbT[o.x + k] & ((1 << SH_SHIFT) - 1);
        const typename MT<M>::V4 gd = g4[e];                   /* d = r_a - r_i */
        const M W = gw[e];
        M Wbar = (M)cacc[(int64_t)a * CP_NACC + CA_EBAR] * pinc;   /* e = sum V W_c */
        if (shep != 0.0) {
            const double *F = cend + (int64_t)a * CP_NEND + CE_F;
            const M sc = Ki * (M)aux[(int64_t)a * ADJ_AUX + 7], sw = sc * W;
            M Ff = 0;
            for (int q = 0; q < c.nd; q++) {
                const M Fq = (M)F[q];
                Ff += Fq * fd0[q];
                fd0b[q].add(-sw * Fq);                           /* fd_a = -sum s fdrag0_i */
            }
            Wbar -= Ff * sc;
            shepb.add(Ff * sw * ishepM);
        }
        const M gw2 = Wbar * gd.w;
        rs[0].add(-gw2 * gd.x);
        rs[1].add(-gw2 * gd.y);
        rs[2].add(-gw2 * gd.z);
    }
    const double shepbv = warp_sum_d(shepb.value());
    if (shepbv != 0.0) {
        /* shep_i = sum_a (m_a / rho_a) W_c(r_ai) */
        const M sb = (M)shepbv;
        for (int k = lane; k < o.y; k += 32) {
            const int e = ixT[o.x + k], a = nbT[o.x + k] & ((1 << SH_SHIFT) - 1);
            const typename MT<M>::V4 gd = g4[e];
            const M gw2 = sb * (M)(mass[a] * aux[(int64_t)a * ADJ_AUX + 7]) * gd.w;
            rs[0].add(-gw2 * gd.x);
            rs[1].add(-gw2 * gd.y);
            rs[2].add(-gw2 * gd.z);
        }
    }
    double fb[3], rr[3];
    for (int q = 0; q < 3; q++) {
        fb[q] = warp_sum_d(fd0b[q].value());
        rr[q] = warp_sum_d(rs[q].value());
    }
    if (lane == 0) {
        double *ai = cacc + i * CP_NACC;
        for (int q = 0; q < c.nd; q++) {
            ai[CA_FD0 + q] += fb[q];
            ai[CA_RS + q] += rr[q];
        }
        ai[CA_SHEP] += shepbv;
    }
}

/* the same terms, fluid side: each fluid particle's position and density
 * adjoints over its DEM partners (coupling table), with the partners'
 * Shepard-sum adjoints from k_cp_cpl_dem */
template <typename M>
__global__ void k_cp_cpl_fluid(DevCfg c, int64_t n, const double *s0, const double *aux, const double *cmid,
                               const double *cend, const double *mass, const int *typ, const int *nb, const int2 *oc,
                               const typename MT<M>::V4 *g4, const M *gw, double *cacc) {
    using Acc = typename MT<M>::Acc;
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    double *ac = cacc + a * CP_NACC;
    const M ebp = (M)(ac[CA_EBAR] * c.por_incr), irho = (M)aux[a * ADJ_AUX + 7], ma = (M)mass[a];
    const M f2d = (M)(c.nd == 2 ? 1.0 / (2.0 * c.dem_radius) : 1.0);
    M F[3] = {0, 0, 0};
    for (int q = 0; q < c.nd; q++) F[q] = (M)cend[a * CP_NEND + CE_F + q];
    Acc rb[3], rhob;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        const int e = o.x + k, i = nb[e] & ((1 << SH_SHIFT) - 1);
        const typename MT<M>::V4 gd = g4[e];                   /* d = r_a - r_i */
        const M W = gw[e];
        M Wbar = ebp;
        const double ishep = cmid[(int64_t)i * CP_NMID + CM_ISHEP];
        if (ishep != 0.0) {
            const double *fd0 = s0 + (int64_t)i * ADJ_NC + AS_FDRAG;
            const M sc = (M)mass[i] * f2d * irho * (M)ishep, sw = sc * W;
            M Ff = 0;
            for (int q = 0; q < c.nd; q++) Ff += F[q] * (M)fd0[q];
            Wbar -= Ff * sc;
            rhob.add(Ff * sw * irho);
        }
        const double sbi = cacc[(int64_t)i * CP_NACC + CA_SHEP];
        if (sbi != 0.0) {
            const M t = (M)sbi * ma * irho;
            rhob.add(-t * W * irho);
            Wbar += t;
        }
        const M gw2 = Wbar * gd.w;
        rb[0].add(gw2 * gd.x);
        rb[1].add(gw2 * gd.y);
        rb[2].add(gw2 * gd.z);
    }
    for (int q = 0; q < c.nd; q++) ac[CA_RS + q] += rb[q].value();
    ac[CA_RHOS] += rhob.value();
}

/* ---- transposed pair tables: each partner's owners ------------------------
 * For a table of owners o -> partners p (entry p | shift code), each
 * partner's owners (key o | shift code, kept for a fixed order) and the
 * index of the pair's entry in the owners' table (its geometry record),
 * sorted by key so that the gathers over them sum in a fixed order.
 * Counting (int atomics), an exclusive scan of the counts, filling,
 * ranking.  Fluid-owned tables (coupling: few partners per owner) take a
 * thread per owner; DEM-owned tables (FPI: ~100 partners per owner) a warp
 * per DEM particle. */
template <bool DEM_OWNERS>
__global__ void k_tr_count(int64_t n, int n_dem, const int *dem_tags, const int *nb, const int2 *oc, int *tcnt) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t o = DEM_OWNERS ? ((t >> 5) < n_dem ? dem_tags[t >> 5] : -1) : (t < n ? t : -1);
    if (o < 0) return;
    const int step = DEM_OWNERS ? 32 : 1;
    const int2 q = oc[o];
    for (int k = DEM_OWNERS ? (threadIdx.x & 31) : 0; k < q.y; k += step)
        atomicAdd(&tcnt[nb[q.x + k] & ((1 << SH_SHIFT) - 1)], 1);
}

template <bool DEM_OWNERS>
__global__ void k_tr_fill(int64_t n, int n_dem, const int *dem_tags, const int *nb, const int2 *oc, const int *toff,
                          int *tfill, int2 *tmp) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t o = DEM_OWNERS ? ((t >> 5) < n_dem ? dem_tags[t >> 5] : -1) : (t < n ? t : -1);
    if (o < 0) return;
    const int step = DEM_OWNERS ? 32 : 1;
    const int2 q = oc[o];
    for (int k = DEM_OWNERS ? (threadIdx.x & 31) : 0; k < q.y; k += step) {
        int sh[3];
        const int p = table_entry(nb[q.x + k], sh);
        for (int d = 0; d < 3; d++) sh[d] = -sh[d];
        tmp[toff[p] + atomicAdd(&tfill[p], 1)] = make_int2((int)o | shift_code(sh), q.x + k);
    }
}

/* DEM partners (long lists): one warp per DEM particle, each entry to its
 * rank among the partner's keys (keys are distinct) */
__global__ void k_tr_rank_dem(int n_dem, const int *dem_tags, const int *toff, const int2 *tmp, int *tnb, int *tix,
                              int2 *toc) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n_dem) return;
    const int64_t p = dem_tags[w];
    const int b0 = toff[p], m = toff[p + 1] - b0;
    for (int k = lane; k < m; k += 32) {
        const int2 v = tmp[b0 + k];
        int r = 0;
        for (int j = 0; j < m; j++) r += (unsigned)tmp[b0 + j].x < (unsigned)v.x;
        tnb[b0 + r] = v.x;
        tix[b0 + r] = v.y;
    }
    if (lane == 0) toc[p] = make_int2(b0, m);
}

/* fluid partners (a few entries each): one thread per particle, insertion
 * sort by key */
__global__ void k_tr_rank_fluid(int64_t n, const int *toff, const int2 *tmp, int *tnb, int *tix, int2 *toc) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int b0 = toff[p], m = toff[p + 1] - b0;
    for (int k = 0; k < m; k++) {
        const int2 v = tmp[b0 + k];
        int r = 0;
        for (int j = 0; j < m; j++) r += (unsigned)tmp[b0 + j].x < (unsigned)v.x;
        tnb[b0 + r] = v.x;
        tix[b0 + r] = v.y;
    }
    toc[p] = make_int2(b0, m);
}

/* exclusive scan of cnt[0, n) into off[0, n], off[n] = total: tiles of
 * SC_TILE counts per block, one block scanning the tile sums */
constexpr int SC_THREADS = 256, SC_PER = 4, SC_TILE = SC_THREADS * SC_PER;

__device__ int block_scan_excl(int v, int *total) {
    __shared__ int ws[SC_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < SC_THREADS / 32 ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < SC_THREADS / 32) ws[lane] = t;
    }
    __syncthreads();
    const int before = wid > 0 ? ws[wid - 1] : 0;
    if (total) *total = ws[SC_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(SC_THREADS) k_sc_tiles(const int *cnt, int64_t n, int *tsum) {
    const int64_t base = (int64_t)blockIdx.x * SC_TILE + threadIdx.x * SC_PER;
    int v = 0;
    for (int k = 0; k < SC_PER; k++)
        if (base + k < n) v += cnt[base + k];
    int total = 0;
    block_scan_excl(v, &total);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

constexpr int SC_SUMS_PER = 16;   /* one block scans up to SC_THREADS * 16 tile sums (4M counts) */
__global__ void __launch_bounds__(SC_THREADS) k_sc_sums(int *tsum, int ntiles) {
    const int base = threadIdx.x * SC_SUMS_PER;
    int v[SC_SUMS_PER], acc = 0;
    for (int k = 0; k < SC_SUMS_PER; k++) {
        v[k] = base + k < ntiles ? tsum[base + k] : 0;
        acc += v[k];
    }
    int run = block_scan_excl(acc, nullptr);
    for (int k = 0; k < SC_SUMS_PER; k++) {
        if (base + k < ntiles) tsum[base + k] = run;
        run += v[k];
    }
}

__global__ void __launch_bounds__(SC_THREADS) k_sc_down(const int *cnt, int64_t n, const int *tsum, int *off) {
    const int64_t base = (int64_t)blockIdx.x * SC_TILE + threadIdx.x * SC_PER;
    int v[SC_PER], acc = 0;
    for (int k = 0; k < SC_PER; k++) {
        v[k] = base + k < n ? cnt[base + k] : 0;
        acc += v[k];
    }
    int run = block_scan_excl(acc, nullptr) + tsum[blockIdx.x];
    for (int k = 0; k < SC_PER; k++) {
        if (base + k < n) off[base + k] = run;
        run += v[k];
        if (base + k == n - 1) off[n] = run;
    }
}

/* the transposed table of (nb, oc) into (tnb, tix, toc); DEM_OWNERS: the
 * owners are the DEM particles (dem_tags), else every particle */
template <bool DEM_OWNERS>
void transpose(sphdem_ctx *c, AdjointData *a, const int *nb, const int2 *oc, TrTable &t) {
    const int64_t n = c->n;
    TrScratch &w = a->trw;
    const int ntiles = (int)((n + SC_TILE - 1) / SC_TILE);
    if (ntiles > SC_THREADS * SC_SUMS_PER) throw std::string("transpose: too many particles");
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(w.cnt, 0, (size_t)n * sizeof(int), c->stream));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(w.fill, 0, (size_t)n * sizeof(int), c->stream));
    const int nd = a->n_dem;
    const int go = DEM_OWNERS ? grid_for((int64_t)std::max(1, nd) * 32, CB) : grid_for(n, CB);
    SPHDEM_LAUNCH(c, "adj_tr_count", k_tr_count<DEM_OWNERS>, go, CB, 0, n, nd, a->dem_tags, nb, oc, w.cnt);
    SPHDEM_LAUNCH(c, "adj_tr_scan", k_sc_tiles, ntiles, SC_THREADS, 0, w.cnt, n, w.tsum);
    SPHDEM_LAUNCH(c, "adj_tr_scan", k_sc_sums, 1, SC_THREADS, 0, w.tsum, ntiles);
    SPHDEM_LAUNCH(c, "adj_tr_scan", k_sc_down, ntiles, SC_THREADS, 0, w.cnt, n, w.tsum, w.off);
    SPHDEM_LAUNCH(c, "adj_tr_fill", k_tr_fill<DEM_OWNERS>, go, CB, 0, n, nd, a->dem_tags, nb, oc, w.off, w.fill, w.tmp);
    if (DEM_OWNERS)
        SPHDEM_LAUNCH(c, "adj_tr_rank", k_tr_rank_fluid, grid_for(n, CB), CB, 0, n, w.off, w.tmp, t.nb, t.ix, t.oc);
    else if (nd > 0)
        SPHDEM_LAUNCH(c, "adj_tr_rank", k_tr_rank_dem, grid_for((int64_t)nd * 32, CB), CB, 0, nd, a->dem_tags, w.off,
                      w.tmp, t.nb, t.ix, t.oc);
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
enum { R_M0 = 0, R_M1, R_M2, R_M3, R_M4, R_E0, R_E1, R_E2, R_O };

/* rm (VAR_H_CORRECTION): the middle record, whose Omega with the end one
 * gives R_O = (Omega_m, Omega_e, kappa_m (set by k_cp_end32_vh), kappa_e),
 * kappa_e = Omegabar_e h / (rho d), Omegabar_e = -Dbar dddt1 / Omega_e */
__global__ void k_cp_pack32(int64_t n, double dt, const double *aux, const double *cmid, const double *s1,
                            const double *adj, const double *mass, const double *hh, const int *typ, float4 *rec,
                            const double *rm, int nd) {
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
    const double Db = aa[AS_DDDT] + hd * aa[AS_DENS];
    rec[R_E2 * n + i] = make_float4((float)x1[AS_VH], (float)x1[AS_VH + 1], (float)x1[AS_VH + 2], (float)Db);
    if (rm) {
        const double ome = x1[AS_OME];
        rec[R_O * n + i] = make_float4((float)rm[i * RM_NC + 3], (float)ome, 0.f,
                                       (float)(-Db * x1[AS_DDDT] / ome * hh[i] / (x[6] * nd)));
    }
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


/* ---- VAR_H_CORRECTION (mixed handles): h = hfac (m / rho_s)^(1/d) follows
 * the density, and every gradient of a particle's sums carries 1 / Omega
 * (calcOmega, sph.h:438-451; gradW, sph.h:331-332):
 *
 *   Omega_x = 1 + h_x S_x / (rho_x d),  S_x = sum_y m_y dW/dh(r_xy, h_x)  (self term included)
 *   middle:  f_x += (1/Omega_x) sum_y [ -m_y (p_x F(r,h_x) + p_y F(r,h_y)) d
 *                                       + c_xy phi_xy w ],
 *            phi = r^2 M / (r^2 + 0.01 hav^2),  M = (F(r,h_x) + F(r,h_y)) / 2
 *   end:     dddt_x = (1/Omega_x) sum_y m_y (w.d) F(r, h_x)
 *   FPI:     W(r / h_b, h_b) with the fluid particle's h
 *
 * with the Wendland C2 kernel W = C h^-d K(q), K = (2-q)^4 (1+2q), and
 * F(r, h) = W'/r = -10 C h^-(d+2) (2-q)^3.  Both phases use h_s and rho_s
 * (the end tail updates them after the continuity pass).  The reverse sweep
 * adds the adjoint of h_s per particle (CA_HB; from the end, middle and FPI
 * sums, and from Omega's own dependence on h), and of Omega_x, which is
 * -Dbar dddt / Omega (end) and -(Pbar.fp + Vbar.fv) / Omega (middle) per
 * particle; its pair terms (dOmega/dr, dOmega/dh) ride in the same pair
 * loops.  Finally rho_s's adjoint takes hbar dh/drho = -hbar h / (d rho). */
template <int ND>
struct KerVH {
    float F, Fr, Fh, Whr, Whh;   /* F, dF/dr, dF/dh, d2W/dh dr, d2W/dh2 */
};

template <int ND>
__device__ __forceinline__ KerVH<ND> ker_vh(float wcon, float r, float ih) {
    KerVH<ND> k = {0.f, 0.f, 0.f, 0.f, 0.f};
    const float q = r * ih;
    if (q > 2.f) return k;
    const float t = 2.f - q, t2 = t * t;
    const float i2 = ipow_nd2<ND>(ih), i3 = i2 * ih;           /* ih^(d+2), ih^(d+3) */
    k.F = -10.f * wcon * i2 * (t2 * t);
    k.Fr = 30.f * wcon * i3 * t2;
    k.Fh = 10.f * wcon * i3 * t2 * ((float)(ND + 2) * t - 3.f * q);
    const float g = t2 * t * ((float)ND * t * (1.f + 2.f * q) - 10.f * q * q);
    const float gp = q * t2 * (30.f * q - 10.f * (float)(ND + 2) * t);
    k.Whr = -wcon * i2 * gp;
    k.Whh = wcon * i2 * ((float)(ND + 1) * g + q * gp);
    return k;
}

/* k_cp_end32 under VAR_H_CORRECTION: continuity with F(r, h_a) / Omega_a and
 * the end Omega's pair terms; then the totals, the adjoints of h_s (CA_HB)
 * and rho_s (CA_RHO) that the end phase gives, and kappa_m */
template <int ND>
__global__ void __launch_bounds__(128) k_cp_end32_vh(DevCfg c, int64_t n, double dt, const int *typ,
                                                     const int *__restrict__ nb, const int2 *__restrict__ oc,
                                                     const double *adj, const double *s1, double *cacc, double *cend,
                                                     float4 *rec) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || !is_fluid(typ[a])) return;
    const float4 *E0 = rec + R_E0 * n, *E1 = rec + R_E1 * n, *E2 = rec + R_E2 * n, *O = rec + R_O * n;
    const float wcon = (float)c.wcon;
    const float4 p0 = E0[a], p1 = E1[a], p2 = E2[a], oa = O[a];
    const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
    const float ma = p1.w, da = p2.w / oa.y, ka = oa.w;   /* delta_a = Dbar / Omega_e, kappa_e */
    Kf rb[ND], wb[ND], hb;
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        int sh[3];
        const int b = table_entry(__ldg(nb + o.x + k), sh);
        float img[3];
        image32<ND>(c, sh, img);
        const float4 q0 = E0[b], q1 = E1[b], q2 = E2[b], ob = O[b];
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
        const float r = sqrtf(r2), ir = 1.f / r;
        const KerVH<ND> ka_ = ker_vh<ND>(wcon, r, p0.w), kb_ = ker_vh<ND>(wcon, r, q0.w);
        const float mb = q1.w, db = q2.w / ob.y, kb = ob.w;
        const float cA = da * mb * ka_.F + db * ma * kb_.F;
        const float cB = (da * mb * ka_.Fr + db * ma * kb_.Fr) * wd + (ka * mb * ka_.Whr + kb * ma * kb_.Whr);
#pragma unroll
        for (int q = 0; q < ND; q++) {
            rb[q].add(cA * w[q] + cB * d[q] * ir);
            wb[q].add(cA * d[q]);
        }
        hb.add(da * mb * wd * ka_.Fh + ka * mb * ka_.Whh);
    }
    const double hd = 0.5 * dt;
    const double *aa = adj + a * ADJ_NC, *x1 = s1 + a * ADJ_NC;
    double *ac = cacc + a * CP_NACC;
    const bool sph = typ[a] == T_SPH;
    double *ce = cend + a * CP_NEND;
    /* Omega_e's own h and rho: Omega - 1 = h S / (rho d) */
    const double rho = rec[R_M2 * n + a].w, ih = p0.w, h = 1.0 / ih;
    const double ombar = (double)ka * rho * ND * ih;
    ac[CA_HB] += hb.value() + ombar * ((double)oa.y - 1.0) * ih +
                 (double)ka * ma * (double)ker_vh<ND>(wcon, 0.f, p0.w).Whh;
    ac[CA_RHO] += -ombar * ((double)oa.y - 1.0) / rho;
    float P[3] = {0.f, 0.f, 0.f}, V[3] = {0.f, 0.f, 0.f};
    double pf = 0.0;   /* Pbar.fp + Vbar.fv of the middle forces */
    for (int q = 0; q < 3; q++) {
        const double rt = aa[AS_R + q] + ac[CA_R1 + q] + (q < ND ? rb[q].value() : 0.0);
        const double vt = aa[AS_VH + q] + ac[CA_VH1 + q] + (q < ND ? wb[q].value() : 0.0) + hd * rt;
        const double F = sph ? aa[AS_F + q] + dt * (vt + aa[AS_V + q]) : 0.0;
        ce[CE_R1 + q] = rt;
        ce[CE_VH1 + q] = vt;
        ce[CE_F + q] = F;
        ce[CE_P + q] = F + ac[CA_FP + q];
        ce[CE_V + q] = sph ? F + ac[CA_FV + q] : 0.0;
        pf += ce[CE_P + q] * x1[AS_FP + q] + ce[CE_V + q] * x1[AS_FV + q];
        P[q] = (float)ce[CE_P + q];
        V[q] = (float)ce[CE_V + q];
    }
    float4 *M3 = rec + R_M3 * n, *M4 = rec + R_M4 * n;
    M3[a] = make_float4(P[0], P[1], P[2], M3[a].w);
    M4[a] = make_float4(V[0], V[1], V[2], M4[a].w);
    /* kappa_m = Omegabar_m h / (rho d), Omegabar_m = -(Pbar.fp + Vbar.fv) / Omega_m */
    rec[R_O * n + a].z = (float)(-pf / (double)oa.x * h / (rho * ND));
}

/* one orientation (x, y) of the middle pair terms under VAR_H_CORRECTION,
 * T = -m_y (p_x F_x + p_y F_y) d + c_xy phi w, against Px, Vx (the adjoints
 * of x's pressure and viscous sums over Omega_x): dT/dd, dT/dw and the
 * adjoints of rho, p and h of x and of y, and of nu */
template <int ND>
struct PairVH {
    float Dd[3], Dw[3], Rx, Ry, Qx, Qy, Hx, Hy, nu;
};

template <int ND>
__device__ __forceinline__ PairVH<ND> force_pair_vh(float nu, float rho0, const float *d, const float *w, float r,
                                                    const KerVH<ND> &kx, const KerVH<ND> &ky, float hav,
                                                    const float *Px, const float *Vx, float my, float rhox,
                                                    float rhoy, float px, float py) {
    PairVH<ND> o;
    float Pd = 0.f, Vw = 0.f;
#pragma unroll
    for (int q = 0; q < ND; q++) {
        Pd = fmaf(Px[q], d[q], Pd);
        Vw = fmaf(Vx[q], w[q], Vw);
    }
    const float ir = 1.f / r, r2 = r * r;
    const float sp = -my * (px * kx.F + py * ky.F), spr = -my * (px * kx.Fr + py * ky.Fr);
    const float Mf = 0.5f * (kx.F + ky.F), Mr = 0.5f * (kx.Fr + ky.Fr);
    const float eta2 = 0.01f * hav * hav, den = 1.f / (r2 + eta2);
    const float phi = Mf * r2 * den;
    const float dphi = Mr * r2 * den + Mf * 2.f * r * eta2 * den * den;
    const float dphh = -Mf * r2 * den * den * 0.01f * hav;      /* dphi/dh through hav (either particle) */
    const float cxy = 2.f * nu * rho0 * my / (rhox * rhoy);
    const float VT = cxy * phi * Vw;
    const float cd = (spr * Pd + cxy * Vw * dphi) * ir;
#pragma unroll
    for (int q = 0; q < ND; q++) {
        o.Dd[q] = sp * Px[q] + cd * d[q];
        o.Dw[q] = cxy * phi * Vx[q];
    }
    o.Rx = -VT / rhox;
    o.Ry = -VT / rhoy;
    o.Qx = -my * kx.F * Pd;
    o.Qy = -my * ky.F * Pd;
    o.Hx = -my * px * kx.Fh * Pd + cxy * Vw * (0.5f * kx.Fh * r2 * den + dphh);
    o.Hy = -my * py * ky.Fh * Pd + cxy * Vw * (0.5f * ky.Fh * r2 * den + dphh);
    o.nu = VT / nu;
    return o;
}

/* k_cp_force32 under VAR_H_CORRECTION: the middle pair terms with F(r, h_x),
 * F(r, h_y) and 1/Omega_x, Omega_m's pair terms, then the EOS and the
 * adjoint of rho_s with h's and Omega_m's parts */
template <int ND>
__global__ void __launch_bounds__(128) k_cp_force32_vh(DevCfg c, int64_t n, const int *typ,
                                                       const int *__restrict__ nb, const int2 *__restrict__ oc,
                                                       const double *adj, const double *aux, const double *cend,
                                                       const float4 *__restrict__ rec, double *cmid, double *cacc,
                                                       double *grads) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float gnu = 0.f;
    if (a < n && is_fluid(typ[a])) {
        const float4 *M0 = rec + R_M0 * n, *M1 = rec + R_M1 * n, *M2 = rec + R_M2 * n, *M3 = rec + R_M3 * n,
                     *M4 = rec + R_M4 * n, *O = rec + R_O * n;
        const float wcon = (float)c.wcon, nu = (float)c.viscosity, rho0 = (float)c.dens;
        const float4 p0 = M0[a], p1 = M1[a], p2 = M2[a], p3 = M3[a], p4 = M4[a], oa = O[a];
        const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
        const float ioa = 1.f / oa.x;
        const float Pa[3] = {p3.x * ioa, p3.y * ioa, p3.z * ioa}, Va[3] = {p4.x * ioa, p4.y * ioa, p4.z * ioa};
        const bool own = p3.x != 0.f || p3.y != 0.f || p3.z != 0.f || p4.x != 0.f || p4.y != 0.f || p4.z != 0.f;
        const float ma = p1.w, ka = oa.z;
        Kf Db[ND], Wb[ND], Rb, Qb, Hb;
        const int2 o = oc[a];
        for (int k = 0; k < o.y; k++) {
            int sh[3];
            const int b = table_entry(__ldg(nb + o.x + k), sh);
            float img[3];
            image32<ND>(c, sh, img);
            const float4 q0 = M0[b], q1 = M1[b], q2 = M2[b], q3 = M3[b], q4 = M4[b], ob = O[b];
            const float pb[3] = {q0.x, q0.y, q0.z}, lb[3] = {q1.x, q1.y, q1.z}, vb[3] = {q2.x, q2.y, q2.z};
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
            const float r = sqrtf(r2), ir = 1.f / r;
            const KerVH<ND> kA = ker_vh<ND>(wcon, r, p0.w), kB = ker_vh<ND>(wcon, r, q0.w);
            const float hav = 0.5f * (p4.w + q4.w);
            const float mb = q1.w;
            if (own) {
                const PairVH<ND> t = force_pair_vh<ND>(nu, rho0, d, w, r, kA, kB, hav, Pa, Va, mb, p2.w, q2.w, p3.w,
                                                       q3.w);
#pragma unroll
                for (int q = 0; q < ND; q++) {
                    Db[q].add(t.Dd[q]);
                    Wb[q].add(t.Dw[q]);
                }
                Rb.add(t.Rx);
                Qb.add(t.Qx);
                Hb.add(t.Hx);
                gnu += t.nu;
            }
            if (q3.x != 0.f || q3.y != 0.f || q3.z != 0.f || q4.x != 0.f || q4.y != 0.f || q4.z != 0.f) {
                const float iob = 1.f / ob.x;
                const float Pb_[3] = {q3.x * iob, q3.y * iob, q3.z * iob}, Vb_[3] = {q4.x * iob, q4.y * iob, q4.z * iob};
                const PairVH<ND> t = force_pair_vh<ND>(nu, rho0, md, mw, r, kB, kA, hav, Pb_, Vb_, ma, q2.w, p2.w,
                                                       q3.w, p3.w);
#pragma unroll
                for (int q = 0; q < ND; q++) {
                    Db[q].add(-t.Dd[q]);
                    Wb[q].add(-t.Dw[q]);
                }
                Rb.add(t.Ry);
                Qb.add(t.Qy);
                Hb.add(t.Hy);
            }
            /* Omega_m's pair terms */
            const float cR = (ka * mb * kA.Whr + ob.z * ma * kB.Whr) * ir;
#pragma unroll
            for (int q = 0; q < ND; q++) Db[q].add(cR * d[q]);
            Hb.add(ka * mb * kA.Whh);
        }
        const double rhoa = aux[a * ADJ_AUX + 6];
        const double eps = cmid[a * CP_NMID + CM_EPS];
        const double x = rhoa / (c.refd * eps), x2 = x * x, x7 = x2 * x2 * x2 * x;
        const double dp_drho = c.prb * (5.0 * x7 + 2.0) / (rhoa * rhoa * rhoa);
        const double dp_deps = -7.0 * c.prb * x7 / (eps * rhoa * rhoa);
        double *ac = cacc + a * CP_NACC;
        const double *aa = adj + a * ADJ_NC, *ea = cend + a * CP_NEND;
        const double Qv = Qb.value();
        /* Omega_m's own h and rho, then h = hfac (m / rho)^(1/d) */
        const double ih = p0.w, h = 1.0 / ih;
        const double ombar = (double)ka * (double)p2.w * ND * ih;
        const double hbar = ac[CA_HB] + Hb.value() + ombar * ((double)oa.x - 1.0) * ih +
                            (double)ka * ma * (double)ker_vh<ND>(wcon, 0.f, p0.w).Whh;
        ac[CA_RHOS] = aa[AS_DENS] + ac[CA_RHO] + Rb.value() + Qv * dp_drho - ombar * ((double)oa.x - 1.0) / rhoa -
                      hbar * h / (ND * rhoa);
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
    const int K = a->K * a->nblk;   /* step slots of the tape store */
    const int64_t n = c->n;
    a->cpl.alloc(K, n);
    a->fpi.alloc(K, n);
    /* one step's transposed coupling and FPI tables, their scratch, the pair
     * geometry of both tables, and the DEM particles' FPI coefficient records */
    const size_t ge = c->cfg.precision == SPHDEM_PREC_MIXED ? sizeof(float) : sizeof(double);
    for (TrTable *t : {&a->cplT, &a->fpiT}) {
        const int64_t cap = t == &a->cplT ? a->cpl.cap : a->fpi.cap;
        SPHDEM_CUDA_CHECK(cudaMalloc(&t->nb, (size_t)cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&t->ix, (size_t)cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&t->oc, (size_t)n * sizeof(int2)));
    }
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->g4_cpl, (size_t)a->cpl.cap * 4 * ge));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->gw_cpl, (size_t)a->cpl.cap * ge));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->g4_fpi, (size_t)a->fpi.cap * 4 * ge));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->gw_fpi, (size_t)a->fpi.cap * ge));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->trw.cnt, (size_t)n * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->trw.fill, (size_t)n * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->trw.off, (size_t)(n + 1) * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->trw.tsum, (size_t)SC_THREADS * SC_SUMS_PER * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->trw.tmp, (size_t)std::max(a->cpl.cap, a->fpi.cap) * sizeof(int2)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->coef, (size_t)n * CP_NCOEF * sizeof(double)));
    if (c->cfg.var_h()) SPHDEM_CUDA_CHECK(cudaMalloc(&a->hs, (size_t)n * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.nb, (size_t)K * a->ct_cap * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.oc, (size_t)K * n * sizeof(int2)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->ct.cnt, (size_t)K * sizeof(int)));
    a->ct.cap = a->ct_cap;
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->rmid, (size_t)K * n * RM_NC * sizeof(double)));
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
    for (int *p : {a->cplT.nb, a->cplT.ix, a->fpiT.nb, a->fpiT.ix, a->trw.cnt, a->trw.fill, a->trw.off, a->trw.tsum})
        cudaFree(p);
    for (void *p : {(void *)a->cplT.oc, (void *)a->fpiT.oc, (void *)a->trw.tmp, (void *)a->coef, a->g4_cpl, a->gw_cpl,
                    a->g4_fpi, a->gw_fpi, (void *)a->hs})
        cudaFree(p);
    a->hs = nullptr;
    a->g4_cpl = a->gw_cpl = a->g4_fpi = a->gw_fpi = nullptr;
    a->cplT = TrTable{};
    a->fpiT = TrTable{};
    a->trw = TrScratch{};
    a->coef = nullptr;
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
    const size_t ocb = (size_t)a->K * c->n * sizeof(int2), sb = (size_t)a->blk * a->K;
    for (PairTable *t : {&a->cpl, &a->fpi, &a->ct}) {
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(t->oc + sb * c->n, 0, ocb, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(t->cnt + sb, 0, a->K * sizeof(int), c->stream));
    }
}

const TapTables *cpl_forward_taps(sphdem_ctx *c, AdjointData *a) {
    if (c->cfg.precision != SPHDEM_PREC_MIXED || c->mx_maxn <= 0) return nullptr;
    /* SPHDEM_ADJ_SCAN_TAPS=1: scan for the tables after each phase as FP64
     * handles do (the tests compare both forms) */
    const char *e = getenv("SPHDEM_ADJ_SCAN_TAPS");
    if (e && e[0] == '1') return nullptr;
    TapTables &t = a->tap;
    t.cpl = TapTable{a->cpl.nb, a->cpl.oc, a->cpl.cnt, a->cpl.cap, 0};
    t.fpi = TapTable{a->fpi.nb, a->fpi.oc, a->fpi.cnt, a->fpi.cap, CP_FPI_PER};
    t.ct = TapTable{a->ct.nb, a->ct.oc, a->ct.cnt, a->ct.cap, ADJ_MAX_CONTACTS};
    t.slot = a->slot;
    return &t;
}

void cpl_taps_middle(sphdem_ctx *c, AdjointData *a) {
    if (!c->tap) {
        k_cp_dpos<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->g, c->n, a->dpos);
        k_cp_cpl_table<<<grid_for(c->n, CB), CB, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, c->n, a->dpos,
                                                                 a->cpl.nb, a->cpl.oc, a->cpl.cnt, a->cpl.cap,
                                                                 a->slot);
    }
    k_cp_tap_r<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->A, c->n, a->rmid, a->slot);
}

void cpl_taps_end(sphdem_ctx *c, AdjointData *a) {
    if (a->n_dem == 0 || c->tap) return;
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
    const size_t sb = (size_t)a->blk * a->K;
    for (int k = 0; k < 3; k++)
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(v.data() + k * a->K, ts[k]->cnt + sb, a->K * sizeof(int),
                                          cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 3; k++)
        for (int j = 0; j < a->K; j++)
            if (v[k * a->K + j] > ts[k]->cap) return true;
    return false;
}

namespace {

/* the coupling passes of the reverse step with pair math in M */
template <typename M>
void cpl_backward_coupling(sphdem_ctx *c, AdjointData *a, int sl, const double *s0, const double *s1, double dt,
                           bool after_forces, const double *hp) {
    using V4 = typename MT<M>::V4;
    const int64_t n = c->n;
    const int nd = a->n_dem;
    const int g = grid_for(n, CB), gd = grid_for((int64_t)std::max(1, nd) * 32, CB);
    const int *nbc = a->cpl.nb + (size_t)sl * a->cpl.cap, *nbf = a->fpi.nb + (size_t)sl * a->fpi.cap;
    const int2 *occ = a->cpl.oc + (size_t)sl * n, *ocf = a->fpi.oc + (size_t)sl * n;
    V4 *g4c = (V4 *)a->g4_cpl, *g4f = (V4 *)a->g4_fpi;
    M *gwc = (M *)a->gw_cpl, *gwf = (M *)a->gw_fpi;
    if (!after_forces) {
        /* pair geometry, the transposed tables, porosity / EOS, Shepard sums,
         * FPI + drag */
        SPHDEM_LAUNCH(c, "adj_geo_cpl", k_cp_geo_cpl<M>, g, CB, 0, c->cfg, n, a->aux, a->typ, nbc, occ, g4c, gwc);
        transpose<false>(c, a, nbc, occ, a->cplT);
        SPHDEM_LAUNCH(c, "adj_por", k_cp_por<M>, g, CB, 0, c->cfg, n, a->aux, a->typ, occ, gwc, a->cmid);
        if (nd == 0) return;
        SPHDEM_LAUNCH(c, "adj_geo_fpi", k_cp_geo_fpi<M>, gd, CB, 0, c->cfg, nd, a->dem_tags, s1, hp, nbf, ocf, g4f,
                      gwf);
        transpose<true>(c, a, nbf, ocf, a->fpiT);
        SPHDEM_LAUNCH(c, "adj_shep", k_cp_shep<M>, gd, CB, 0, nd, a->dem_tags, a->aux, a->mass, a->cplT.nb, a->cplT.ix,
                      a->cplT.oc, gwc, a->cmid);
        SPHDEM_LAUNCH(c, "adj_fpi_dem", k_cp_fpi<M>, gd, CB, 0, c->cfg, nd, a->dem_tags, dt, s1, a->aux, a->cmid,
                      a->mass, nbf, ocf, g4f, gwf, a->adj, a->cacc, a->coef, a->grads);
        if (c->cfg.var_h())
            SPHDEM_LAUNCH(c, "adj_fpi_fluid", (k_cp_fpi_fluid<M, true>), g, CB, 0, n, c->cfg.nd, s1, a->aux, a->cmid,
                          a->mass, a->typ, a->fpiT.nb, a->fpiT.ix, a->fpiT.oc, g4f, gwf, a->coef, a->cacc, hp,
                          c->cfg.wcon);
        else
            SPHDEM_LAUNCH(c, "adj_fpi_fluid", (k_cp_fpi_fluid<M, false>), g, CB, 0, n, c->cfg.nd, s1, a->aux, a->cmid,
                          a->mass, a->typ, a->fpiT.nb, a->fpiT.ix, a->fpiT.oc, g4f, gwf, a->coef, a->cacc, hp,
                          c->cfg.wcon);
        return;
    }
    /* porosity, DEM -> fluid drag and Shepard terms, after the forces gave
     * the adjoints of e and f */
    if (nd > 0)
        SPHDEM_LAUNCH(c, "adj_cpl_dem", k_cp_cpl_dem<M>, gd, CB, 0, c->cfg, nd, a->dem_tags, s0, a->aux, a->cmid,
                      a->cend, a->mass, a->cplT.nb, a->cplT.ix, a->cplT.oc, g4c, gwc, a->cacc);
    SPHDEM_LAUNCH(c, "adj_cpl_fluid", k_cp_cpl_fluid<M>, g, CB, 0, c->cfg, n, s0, a->aux, a->cmid, a->cend, a->mass,
                  a->typ, nbc, occ, g4c, gwc, a->cacc);
}

}  // namespace

void cpl_backward_step(sphdem_ctx *c, AdjointData *a, int j, double dt) {
    const int64_t n = c->n;
    /* step j of the segment in tape block a->blk */
    const size_t stb = (size_t)a->blk * (a->K + 1);
    const double *s0 = a->seg + (stb + j - 1) * n * ADJ_NC, *s1 = a->seg + (stb + j) * n * ADJ_NC;
    const int sl = a->blk * a->K + j - 1;
    const double *rm = a->rmid + (size_t)sl * n * RM_NC;
    auto nbp = [&](const PairTable &t) { return t.nb + (size_t)sl * t.cap; };
    auto ocp = [&](const PairTable &t) { return t.oc + (size_t)sl * n; };
    const int *nbm = a->nb_mid + (size_t)sl * a->pair_cap, *nbe = a->nb_end + (size_t)sl * a->pair_cap;
    const int2 *ocm = a->oc_mid + (size_t)sl * n, *oce = a->oc_end + (size_t)sl * n;
    const int g = grid_for(n, CB), g256 = grid_for(n, 256);
    const bool mixed = a->crec != nullptr, vh = c->cfg.var_h();
    /* the step's smoothing lengths: h_s under VAR_H_CORRECTION, else constant */
    const double *hp = vh ? a->hs : a->hh;
    cudaStream_t st = c->stream;
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->cacc, 0, (size_t)n * CP_NACC * sizeof(double), st));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->cmid, 0, (size_t)n * CP_NMID * sizeof(double), st));
    SPHDEM_LAUNCH(c, "adj_pre", k_cp_pre, g256, 256, 0, n, dt, s0, rm, a->typ, a->aux, a->mass, a->hh,
                  vh ? a->hs : nullptr, c->cfg.hfac, c->cfg.nd);
    if (mixed) cpl_backward_coupling<float>(c, a, sl, s0, s1, dt, false, hp);
    else cpl_backward_coupling<double>(c, a, sl, s0, s1, dt, false, hp);
    SPHDEM_LAUNCH(c, "adj_contacts", k_cp_dem, g, CB, 0, c->cfg, n, dt, s1, a->aux, a->mass, a->rad, a->typ,
                  nbp(a->ct), ocp(a->ct), a->adj, a->cacc, a->grads);
    if (mixed) {
        SPHDEM_LAUNCH(c, "adj_pack32", k_cp_pack32, g256, 256, 0, n, dt, a->aux, a->cmid, s1, a->adj, a->mass, hp,
                      a->typ, a->crec, vh ? rm : nullptr, c->cfg.nd);
#define L_(ND)                                                                                                   \
    do {                                                                                                         \
        if (vh) {                                                                                                \
            SPHDEM_LAUNCH(c, "adj_end32", k_cp_end32_vh<ND>, g, CB, 0, c->cfg, n, dt, a->typ, nbe, oce, a->adj,   \
                          s1, a->cacc, a->cend, a->crec);                                                         \
            SPHDEM_LAUNCH(c, "adj_force32", k_cp_force32_vh<ND>, g, CB, 0, c->cfg, n, a->typ, nbm, ocm, a->adj,   \
                          a->aux, a->cend, a->crec, a->cmid, a->cacc, a->grads);                                  \
        } else {                                                                                                 \
            SPHDEM_LAUNCH(c, "adj_end32", k_cp_end32<ND>, g, CB, 0, c->cfg, n, dt, a->typ, nbe, oce, a->adj,      \
                          a->cacc, a->cend, a->crec);                                                             \
            SPHDEM_LAUNCH(c, "adj_force32", k_cp_force32<ND>, g, CB, 0, c->cfg, n, a->typ, nbm, ocm, a->adj,      \
                          a->aux, a->cend, a->crec, a->cmid, a->cacc, a->grads);                                  \
        }                                                                                                        \
    } while (0)
        if (c->cfg.nd == 3) L_(3);
        else if (c->cfg.nd == 2) L_(2);
        else L_(1);
#undef L_
        cpl_backward_coupling<float>(c, a, sl, s0, s1, dt, true, hp);
    } else {
        SPHDEM_LAUNCH(c, "adj_end", k_cp_end, g, CB, 0, c->cfg, n, dt, s1, a->mass, a->hh, a->typ, nbe, oce, a->adj,
                      a->cacc, a->cend);
        SPHDEM_LAUNCH(c, "adj_force", k_cp_force, g, CB, 0, c->cfg, n, a->aux, a->mass, a->hh, a->typ, nbm, ocm,
                      a->adj, a->cend, a->cmid, a->cacc, a->grads);
        cpl_backward_coupling<double>(c, a, sl, s0, s1, dt, true, hp);
    }
    SPHDEM_LAUNCH(c, "adj_assemble", k_cp_assemble, g256, 256, 0, n, dt, a->typ, a->cacc, a->cend, a->cmid, a->adj);
}

}  // namespace sphdem
