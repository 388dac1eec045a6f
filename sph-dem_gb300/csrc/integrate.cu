/*
 * Elementwise parts of a step: the integrator functors of sphIncompress.h
 * (driftR 620-641, driftRAndKick 643-676, driftRest 678-704, kick 706-742,
 * initSumsMiddle 744-763, initSumsEnd 765-767), the dt choice of
 * sphIncompress.cpp:126-154, and the device built-ins of the case hooks
 * (gravity, planar DEM walls and DEM freezing in the pattern of
 * sediment3D/customSim.cpp:5-113).
 *
 * Each launch fuses every per-particle functor the reference runs back to
 * back in one phase, so a phase touches each live field once.  All of them
 * are HBM-bound: bytes per particle = the rows read + written below.
 */
#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 256;

__global__ void k_globals_op(DevCfg c, DevGlobals *g, int op) {
    if (threadIdx.x || blockIdx.x) return;
    switch (op) {
        case OP_MIDDLE_BEGIN:
            g->new_dt = g->maxdt;
            g->new_dt_bits = dbits(g->maxdt);
            break;
        case OP_SET_DT: {
            double nd = __longlong_as_double((long long)g->new_dt_bits);
            if (c.liq_dem()) {
                nd = fmin(nd, c.liq_dem_timestep);
                if (g->time > c.time_drop) nd = fmin(nd, c.dem_timestep);
            }
            g->new_dt = nd;
            g->old_dt = g->dt;
            if (c.flags & SPHDEM_F_FIXED_DT) g->dt = g->maxdt;
            else g->dt = nd;
            break;
        }
        case OP_END_BEGIN:
            g->dem_dt = g->maxdt;
            break;
        case OP_STEP_INC:
            g->step += 1;
            break;
    }
}

__device__ __forceinline__ void eos(const DevCfg &c, const DevState &s, int64_t i) {
    const double dens = s.row(FD_DENS)[i];
    double press;
    if (c.liq_dem()) {
        const double x = dens * recip(c, c.refd * s.row(FD_POR)[i]);
        double xg;
        if (c.gamma == 7.0) {
            const double x2 = x * x;
            xg = x2 * x2 * x2 * x;
        } else {
            xg = pow(x, c.gamma);
        }
        press = c.prb * (xg - 1.0);
    } else {
        const double x = dens / c.refd;
        const double x2 = x * x;
        press = c.prb * (x2 * x2 * x2 * x - 1.0);
    }
    const double rd = recip(c, dens);
    s.row(FD_PRESS)[i] = press;
    s.row(FD_PDR2)[i] = press * (rd * rd);
}

/* start(): driftRAndKick + driftRest + initSumsMiddle for sph/sphBoundary,
 * driftR for dem, time += dt/2 (sphIncompress.cpp:3-38, no density re-init) */
__global__ void k_start(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double dt = g->dt;
    if (i == 0) g->time = g->time + dt / 2;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    const double hd = dt / 2;
    if (is_sph_or_sphb(t)) {
        for (int d = 0; d < c.nd; d++) {
            double *r = s.row(FD_R + d), *vh = s.row(FD_VHAT + d);
            r[i] += hd * vh[i];
            if (t != T_SPHB) {
                double *v = s.row(FD_V + d), *f = s.row(FD_F + d);
                s.row(FD_V0 + d)[i] = v[i];
                s.row(FD_VHAT0 + d)[i] = vh[i];
                v[i] += hd * f[i];
                vh[i] += hd * f[i];
            }
        }
        double *dens = s.row(FD_DENS);
        dens[i] += hd * s.row(FD_DDDT)[i];
        if (!(c.flags & SPHDEM_F_CONST_H)) {
            s.row(FD_H)[i] = smoothing_length(c, s.row(FD_MASS)[i] * recip(c, dens[i]));
            h_derived(c, s, i);
        }
        for (int d = 0; d < 3; d++) {
            s.row(FD_F + d)[i] = 0.0;
            s.row(FD_FP + d)[i] = 0.0;
            s.row(FD_FV + d)[i] = 0.0;
            s.row(FD_FB + d)[i] = 0.0;
        }
    } else if (c.liq_dem() && t == T_DEM) {
        for (int d = 0; d < c.nd; d++) s.row(FD_R + d)[i] += hd * s.row(FD_VHAT + d)[i];
    }
}

/* beforeMiddle built-in: gravity on type sph (sediment3D/customSim.cpp:90-95) */
__global__ void k_hook_before_middle(DevCfg c, DevState s, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (s.irow(FI_IAM)[i] != T_SPH) return;
    for (int d = 0; d < c.nd; d++)
        if (c.g_sph[d] != 0.0) s.row(FD_F + d)[i] += c.g_sph[d];
}

/* middle() after the force loop: kick sph/sphBoundary with (oldDt+dt)/2,
 * initSumsEnd, then for dem driftRAndKick + initSumsMiddle
 * (sphIncompress.cpp:157-164) */
__global__ void k_middle_tail(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    const double dt = g->dt, old_dt = g->old_dt;
    if (is_sph_or_sphb(t)) {
        if (t == T_SPH) {
            const double k = 0.5 * old_dt + 0.5 * dt;
            const bool damp = g->time < c.damptime;
            for (int d = 0; d < c.nd; d++) {
                const double f = s.row(FD_F + d)[i];
                double v = s.row(FD_V0 + d)[i] + k * f;
                double vh = s.row(FD_VHAT0 + d)[i] + k * f;
                if (damp) {
                    v *= 0.98;
                    vh *= 0.98;
                }
                s.row(FD_V + d)[i] = v;
                s.row(FD_VHAT + d)[i] = vh;
            }
        }
        s.row(FD_DDDT)[i] = 0.0;
    } else if (c.liq_dem() && t == T_DEM) {
        const double hd = dt / 2;
        for (int d = 0; d < c.nd; d++) {
            double *r = s.row(FD_R + d), *v = s.row(FD_V + d), *vh = s.row(FD_VHAT + d);
            const double f = s.row(FD_F + d)[i];
            r[i] += hd * vh[i];
            s.row(FD_V0 + d)[i] = v[i];
            s.row(FD_VHAT0 + d)[i] = vh[i];
            v[i] += hd * f;
            vh[i] += hd * f;
        }
        for (int d = 0; d < 3; d++) {
            s.row(FD_F + d)[i] = 0.0;
            s.row(FD_FP + d)[i] = 0.0;
            s.row(FD_FV + d)[i] = 0.0;
            s.row(FD_FB + d)[i] = 0.0;
        }
    }
}

/* end(): driftR for sph/sphBoundary, time += dt/2 (sphIncompress.cpp:169-183) */
__global__ void k_end_drift(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double dt = g->dt;
    if (i == 0) {
        g->time = g->time + dt / 2;
        if (c.liq_dem()) g->dem_dt = g->maxdt;
    }
    if (i >= n) return;
    if (!is_sph_or_sphb(s.irow(FI_IAM)[i])) return;
    for (int d = 0; d < c.nd; d++) s.row(FD_R + d)[i] += (dt / 2) * s.row(FD_VHAT + d)[i];
}

/* end() tail: dem kick(dt/2,dt/2) (sphIncompress.cpp:239), driftRest for
 * sph/sphBoundary (245) and calcEnergies (249, sphIncompress.h:769-781): EOS
 * refresh, elastic energy u += dt pdr2 dddt, and for sph the viscous energy
 * eViscF += dt (-vhat . fv) */
__global__ void k_end_tail(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    const double dt = g->dt;
    if (c.liq_dem() && t == T_DEM) {
        const double k = 0.5 * dt + 0.5 * dt;
        const bool damp = g->time < c.damptime;
        const bool block = c.flags & SPHDEM_F_DEM_BLOCK;
        for (int d = 0; d < c.nd; d++) {
            if (block) s.row(FD_F + d)[i] = g->dem_avf[d];   /* setAvForce, sphIncompress.h:112-114 */
            const double f = s.row(FD_F + d)[i];
            double v = s.row(FD_V0 + d)[i] + k * f;
            double vh = s.row(FD_VHAT0 + d)[i] + k * f;
            if (damp) {
                v *= 0.98;
                vh *= 0.98;
            }
            s.row(FD_V + d)[i] = v;
            s.row(FD_VHAT + d)[i] = vh;
        }
    } else if (is_sph_or_sphb(t)) {
        double *dens = s.row(FD_DENS);
        dens[i] += (dt / 2) * s.row(FD_DDDT)[i];
        if (!(c.flags & SPHDEM_F_CONST_H)) {
            s.row(FD_H)[i] = smoothing_length(c, s.row(FD_MASS)[i] * recip(c, dens[i]));
            h_derived(c, s, i);
        }
        eos(c, s, i);
        const double dudt = s.row(FD_PDR2)[i] * s.row(FD_DDDT)[i];
        s.row(FD_DUDT)[i] = dudt;
        s.row(FD_U)[i] += dt * dudt;
        if (t == T_SPH) {
            double w = 0.0;
            for (int d = 0; d < c.nd; d++) w += s.row(FD_VHAT + d)[i] * s.row(FD_FV + d)[i];
            s.row(FD_DEVISCF)[i] = -w;
            s.row(FD_EVISCF)[i] += dt * (-w);
        }
    }
}

/* DEM_BLOCK: calcAvForce over the DEM particles (sphIncompress.h:107-110) and
 * the mean (sphIncompress.cpp:232-236).  One block, a fixed reduction tree:
 * the same sum on every run. */
constexpr int AVF_BLK = 1024;
__global__ void __launch_bounds__(AVF_BLK) k_dem_block(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    __shared__ double sh[4][AVF_BLK / 32];
    double acc[4] = {0, 0, 0, 0};
    for (int64_t i = threadIdx.x; i < n; i += AVF_BLK) {
        if (s.irow(FI_IAM)[i] != T_DEM) continue;
        for (int d = 0; d < c.nd; d++) acc[d] += s.row(FD_F + d)[i];
        acc[3] += 1.0;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < 4; k++) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++)
            for (int j = 0; j < AVF_BLK / 32; j++) t[k] += sh[k][j];
        for (int d = 0; d < 3; d++) g->dem_avf[d] = t[3] > 0 ? t[d] / t[3] : 0.0;
    }
}

__device__ __forceinline__ double dem_radius(const DevCfg &c, const DevState &s, int64_t i) {
    const double r = s.row(FD_RADIUS)[i];
    return r > 0.0 ? r : c.dem_radius;
}

/* beforeEnd built-ins for dem: gravity, planar walls, freeze */
__global__ void k_hook_before_end(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!c.liq_dem() || s.irow(FI_IAM)[i] != T_DEM) return;
    for (int d = 0; d < c.nd; d++)
        if (c.g_dem[d] != 0.0) s.row(FD_F + d)[i] += c.g_dem[d];
    const double R = dem_radius(c, s, i), m = s.row(FD_MASS)[i];
    for (int w = 0; w < c.n_walls; w++) {
        double dist = 0.0, vn = 0.0;
        double dd[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) {
            dd[d] = s.row(FD_R + d)[i] - c.wall_p[w][d];
            vv[d] = s.row(FD_VHAT + d)[i];
        }
        if (c.nd == 3) {
            dist = dd[0] * c.wall_n[w][0] + (dd[1] * c.wall_n[w][1] + dd[2] * c.wall_n[w][2]);
            vn = vv[0] * c.wall_n[w][0] + (vv[1] * c.wall_n[w][1] + vv[2] * c.wall_n[w][2]);
        } else {
            dist = dd[0] * c.wall_n[w][0] + dd[1] * c.wall_n[w][1];
            vn = vv[0] * c.wall_n[w][0] + vv[1] * c.wall_n[w][1];
        }
        const double overlap = R - dist;
        if (overlap > 0.0) {
            const double sN = c.dem_k * overlap + c.dem_gamma * (-vn);
            for (int d = 0; d < c.nd; d++) {
                const double fN = (sN * c.wall_n[w][d]) / m;
                s.row(FD_FB + d)[i] += fN;
                s.row(FD_F + d)[i] += fN;
            }
        }
    }
    if (g->time <= c.freeze_until)
        for (int d = 0; d < 3; d++) {
            s.row(FD_F + d)[i] = 0.0;
            s.row(FD_V + d)[i] = 0.0;
            s.row(FD_VHAT + d)[i] = 0.0;
        }
}

__global__ void k_hook_after_end(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!c.liq_dem() || s.irow(FI_IAM)[i] != T_DEM) return;
    if (g->time <= c.freeze_until)
        for (int d = 0; d < 3; d++) {
            s.row(FD_F + d)[i] = 0.0;
            s.row(FD_V + d)[i] = 0.0;
            s.row(FD_VHAT + d)[i] = 0.0;
        }
}

__global__ void k_h_derived(DevCfg c, DevState s, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (s.irow(FI_IAM)[i] == T_DEAD) return;
    h_derived(c, s, i);
}

}  // namespace

void run_h_derived(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "h_derived", k_h_derived, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->n);
}

void globals_op(sphdem_ctx *c, int op) {
    SPHDEM_LAUNCH(c, "globals_op", k_globals_op, 1, 32, 0, c->cfg, c->g, op);
}
void run_start(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "start", k_start, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_hook_before_middle(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "hook_before_middle", k_hook_before_middle, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->n);
}
void run_middle_tail(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "middle_tail", k_middle_tail, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_end_drift(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "end_drift", k_end_drift, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_dem_block(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "dem_block", k_dem_block, 1, AVF_BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_end_tail(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "end_tail", k_end_tail, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_hook_before_end(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "hook_before_end", k_hook_before_end, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}
void run_hook_after_end(sphdem_ctx *c) {
    SPHDEM_LAUNCH(c, "hook_after_end", k_hook_after_end, grid_for(c->n, BLK), BLK, 0, c->cfg, c->A, c->g, c->n);
}

}  // namespace sphdem
