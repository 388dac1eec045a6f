/*
 * Adjoint of the step (reverse mode), with step checkpointing.
 *
 * sphdem_adjoint_forward runs the steps through the ordinary path and keeps
 * the state (r, v, vh, f, dens, dddt in tag order) and the step globals every
 * `ckpt_every` steps.  sphdem_adjoint_backward walks the segments from the
 * last: it restores the segment's checkpoint into the handle, replays its
 * steps while keeping every step's state and the pairs the step used (the
 * same exact FP64 predicate, particle.h:236-238), then applies the step's
 * vector-Jacobian product in reverse order.  Replays are bit-identical to the
 * first forward pass (the bucket order is a deterministic function of the
 * positions), so the gradients are those of the computed trajectory.  Two
 * step families are differentiated.
 *
 * DEM (handles whose particles are all DEM: LIQ_DEM without fluid, the
 * granular settling configuration).  The step (k_start, k_middle_tail,
 * k_hook_before_end, the contact pass of the end phase, k_end_tail;
 * sphIncompress.cpp:3-251 with the sediment3D hooks) reduces to
 *
 *   r1  = r0 + dt vh0
 *   vhm = vh0 + dt/2 f0                       (middle kick, seen by the dashpots)
 *   f1  = g + walls(r1, vhm) + contacts(r1, vhm)
 *   vh1 = vh0 + dt f1,   v1 = v0 + dt f1
 *
 * with linear spring-dashpot contacts (calcDEMContacts, sph.h:1676-1706):
 * f_a += (k d + gamma d') n / m_a, d = Ra + Rb - |u|, n = u/|u|,
 * d' = -(vh_a - vh_b).n, u = r_a - image(r_b), and planar walls
 * (sediment3D customSim.cpp:67-81): f += (k (R - (r-p).n_w) - gamma vh.n_w) n_w / m.
 * Gradients: dem_k, dem_gamma, initial r / v / vh.  Contact pairs are
 * scattered with FP64 atomics.
 *
 * SPH (weakly compressible fluid with fixed sphBoundary particles: types SPH
 * and SPHB only, artificial viscosity, constant h, no anticlumping, no
 * VAR_H_CORRECTION, no periodic axes; the dam break).  With hd = dt/2 and
 * tag-order state, for an SPH particle (an SPHB particle is never kicked:
 * vh_s = vh1 = vh0, v1 = v0, and its force is read by nothing):
 *
 *   r_s = r0 + hd vh0,  vh_s = vh0 + hd f0,  rho_s = rho0 + hd dddt0      (start, sphIncompress.h:643-704)
 *   pdr2_s = PRB((rho_s/refd)^7 - 1) / rho_s^2                           (sphIncompress.h:863-896)
 *   f1  = g + sum_b [m_b Pi_ab - m_b (pdr2_a + pdr2_b)] G_ab d_ab         (calcForce, sph.h:579-734)
 *   vh1 = vh0 + dt f1,  v1 = v0 + dt f1                                  (kick, sphIncompress.h:706-742)
 *   r1  = r_s + hd vh1                                                   (driftR)
 *   dddt1 = sum_b m_b (vh1_a - vh1_b) . G_ab d_ab                        (calcDddtDudt, sphIncompress.h:783-851)
 *   rho1 = rho_s + hd dddt1                                              (driftRest)
 *
 * where d_ab = r_a - r_b, G_ab = (F(r, h_a) + F(r, h_b)) / 2 with the
 * Wendland C2 gradient factor F(r, h) = -10 C (2 - r/h)^3 / h^(d+2), and the
 * artificial viscosity Pi_ab = alpha s (2 c0 - 4 s) / (rho_a + rho_b) for
 * s = d.(vh_a - vh_b) / r < 0 (sph.h:633-646).  The middle sums run over the
 * pairs of the middle rebuild (at r_s), the continuity sum over those of the
 * end rebuild (at r1).  Gradients: alpha (reported as the viscosity
 * gradient), initial r / v / vh.  Every ordered pair (a, b) is listed with
 * its reverse (b, a), so the reverse passes gather, per particle, the terms
 * of its own pairs and those of its partners' pairs: no atomics, and the
 * result does not depend on the launch order.
 */
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint.cuh"

namespace sphdem {

void adjoint_free(sphdem_ctx *c) {
    AdjointData *a = c->adj;
    if (!a) return;
    for (double *p : a->ckpt) cudaFree(p);
    for (cudaGraphExec_t g : a->graph)
        if (g) cudaGraphExecDestroy(g);
    cudaFree(a->seg);
    cudaFree(a->pairs);
    cudaFree(a->pair_cnt);
    cudaFree(a->adj);
    cudaFree(a->racc);
    cudaFree(a->vmacc);
    cudaFree(a->fbar);
    cudaFree(a->mass);
    cudaFree(a->rad);
    cudaFree(a->typ);
    cudaFree(a->hh);
    cudaFree(a->nb_mid);
    cudaFree(a->nb_end);
    cudaFree(a->oc_mid);
    cudaFree(a->oc_end);
    cudaFree(a->cnt_end);
    cudaFree(a->slot);
    cudaFree(a->aux);
    cudaFree(a->rec);
    cudaFree(a->grads);
    cpl_free(a);
    delete a;
    c->adj = nullptr;
}

namespace {

constexpr int ABLK = 256;

/* with slot: the state after step *slot of the tape store, whose blocks of K
 * steps each hold K + 1 states (the block's first state, then one per step) */
__global__ void k_save(DevState s, int64_t n, double *dst, const int *slot, int K) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (slot) dst += (int64_t)(*slot + 1 + *slot / K) * n * ADJ_NC;
    double *o = dst + (int64_t)s.irow(FI_TAG)[k] * ADJ_NC;
    for (int d = 0; d < 3; d++) {
        o[d] = s.row(FD_R + d)[k];
        o[3 + d] = s.row(FD_V + d)[k];
        o[6 + d] = s.row(FD_VHAT + d)[k];
        o[9 + d] = s.row(FD_F + d)[k];
    }
    o[AS_DENS] = s.row(FD_DENS)[k];
    o[AS_DDDT] = s.row(FD_DDDT)[k];
    for (int d = 0; d < 3; d++) {
        o[AS_FDRAG + d] = s.row(FD_FDRAG + d)[k];
        o[AS_FP + d] = s.row(FD_FP + d)[k];
        o[AS_FV + d] = s.row(FD_FV + d)[k];
    }
    o[AS_OME] = s.row(FD_OMEGA)[k];
}

__global__ void k_restore(DevState s, int64_t n, const double *src) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double *o = src + (int64_t)s.irow(FI_TAG)[k] * ADJ_NC;
    for (int d = 0; d < 3; d++) {
        s.row(FD_R + d)[k] = o[d];
        s.row(FD_V + d)[k] = o[3 + d];
        s.row(FD_VHAT + d)[k] = o[6 + d];
        s.row(FD_F + d)[k] = o[9 + d];
    }
    s.row(FD_DENS)[k] = o[AS_DENS];
    s.row(FD_DDDT)[k] = o[AS_DDDT];
    for (int d = 0; d < 3; d++) {
        s.row(FD_FDRAG + d)[k] = o[AS_FDRAG + d];
        s.row(FD_FP + d)[k] = o[AS_FP + d];
        s.row(FD_FV + d)[k] = o[AS_FV + d];
    }
}

__global__ void k_slot_inc(int *slot) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *slot += 1;
}

__global__ void k_slot_set(int *slot, int v) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *slot = v;
}

__global__ void k_save_const(DevCfg c, DevState s, int64_t n, double *mass, double *rad, int *typ, double *hh) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = s.irow(FI_TAG)[k];
    mass[t] = s.row(FD_MASS)[k];
    /* radius, or -1 for a particle that is not (or no longer) DEM */
    rad[t] = s.irow(FI_IAM)[k] != T_DEM ? -1.0 : (s.row(FD_RADIUS)[k] > 0 ? s.row(FD_RADIUS)[k] : c.dem_radius);
    typ[t] = s.irow(FI_IAM)[k];
    hh[t] = s.row(FD_H)[k];
}

/* the contact pairs the end phase just used: DEM neighbours (exact FP64
 * predicate, particle.h:236-238) with a positive overlap, in tag indices */
__global__ void k_contacts(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g, int64_t n,
                           int4 *pairs, int *cnt, int cap) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n || s.irow(FI_IAM)[a] != T_DEM) return;
    const int nsc = g->n_sph_cells;
    int cc[3] = {0, 0, 0};
    {
        int key = skey[a] - nsc;
        for (int d = c.nd - 1; d >= 0; d--) {
            cc[d] = key % c.ddims[d];
            key /= c.ddims[d];
        }
    }
    const double Ra = s.row(FD_RADIUS)[a] > 0 ? s.row(FD_RADIUS)[a] : c.dem_radius;
    const double ha = s.row(FD_H)[a];
    int o[3] = {0, 0, 0};
    for (o[0] = -1; o[0] <= 1; o[0]++)
        for (o[1] = (c.nd > 1 ? -1 : 0); o[1] <= (c.nd > 1 ? 1 : 0); o[1]++)
            for (o[2] = (c.nd > 2 ? -1 : 0); o[2] <= (c.nd > 2 ? 1 : 0); o[2]++) {
                int sh[3] = {0, 0, 0}, lin = 0;
                bool ok = true;
                for (int d = 0; d < c.nd; d++) {
                    int t = cc[d] + o[d];
                    if (t < 0) {
                        ok = ok && c.periodic[d];
                        t += c.ddims[d];
                        sh[d] = -1;
                    } else if (t >= c.ddims[d]) {
                        ok = ok && c.periodic[d];
                        t -= c.ddims[d];
                        sh[d] = 1;
                    }
                    lin = lin * c.ddims[d] + t;
                }
                if (!ok) continue;
                const bool shifted = sh[0] || sh[1] || sh[2];
                for (int b = start[nsc + lin]; b < start[nsc + lin + 1]; b++) {
                    if (b == a && !shifted) continue;
                    if (s.irow(FI_IAM)[b] != T_DEM) continue;
                    if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) continue;
                    double dx[3] = {0, 0, 0};
                    for (int d = 0; d < c.nd; d++)
                        dx[d] = dsub(s.row(FD_R + d)[a], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
                    const double r2 = exact_len2(dx, c.nd);
                    const double hb = s.row(FD_H)[b];
                    const double t2 = 2.0 * (ha > hb ? ha : hb);
                    if (!(r2 <= dmul(t2, t2))) continue;
                    const double Rb = s.row(FD_RADIUS)[b] > 0 ? s.row(FD_RADIUS)[b] : c.dem_radius;
                    if (!((Ra + Rb) - sqrt(r2) > 0.0)) continue;
                    const int slot = atomicAdd(cnt, 1);
                    if (slot < cap)
                        pairs[slot] = make_int4(s.irow(FI_TAG)[a], s.irow(FI_TAG)[b],
                                                (sh[0] + 1) | ((sh[1] + 1) << 2) | ((sh[2] + 1) << 4), 0);
                }
            }
}

/* SPH pairs of particle a in the current buckets: every SPH/SPHB b with
 * |r_a - image(r_b)|^2 <= (2 max(h_a, h_b))^2 (particle.h:236-238, FP64
 * without contraction); with WRITE, the first `room` of them are written as
 * tag_b | shift code << 26.  Returns the count. */
template <bool WRITE>
__device__ __forceinline__ int sph_pairs_of(const DevCfg &c, const DevState &s, const int *start, const int *skey,
                                            const int *dims, int64_t a, int *out, int64_t room) {
    const CellCoord cc = decode_cell(skey[a], dims, c.nd);
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ha = s.row(FD_H)[a];
    int k = 0;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
            for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                int sh[3];
                const int lin = neighbour_cell(cc, ox, oy, oz, dims, c.periodic, c.nd, sh);
                if (lin < 0) continue;
                const bool shifted = sh[0] || sh[1] || sh[2];
                for (int b = start[lin]; b < start[lin + 1]; b++) {
                    if (b == a && !shifted) continue;
                    if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) continue;
                    if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) continue;
                    double dx[3] = {0, 0, 0};
                    for (int d = 0; d < c.nd; d++)
                        dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
                    const double r2 = exact_len2(dx, c.nd);
                    const double hb = s.row(FD_H)[b];
                    const double t2 = 2.0 * (ha > hb ? ha : hb);
                    if (!(r2 <= dmul(t2, t2))) continue;
                    if (WRITE && k < room)
                        out[k] = s.irow(FI_TAG)[b] |
                                 (((sh[0] + 1) | ((sh[1] + 1) << 2) | ((sh[2] + 1) << 4)) << SH_SHIFT);
                    k++;
                }
            }
    return k;
}

/* The SPH pair list of the current buckets, grouped by particle:
 * nb[slot * cap + ...] = partner entries, oc[slot * n + tag_a] = (offset,
 * count), cnt[slot] = entries used.  One atomic per warp reserves the warp's
 * entries.  With nb == nullptr only cnt[0] is counted.  An overflowing
 * particle records count 0 and the caller sees cnt > cap. */
__global__ void k_sph_pairs(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g, int64_t n,
                            int *nb, int2 *oc, int *cnt, int64_t cap, const int *slot) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int dims[3] = {g->sdims[0], g->sdims[1], g->sdims[2]};
    const bool live = a < n && is_sph_or_sphb(s.irow(FI_IAM)[a]);
    const int j = slot ? *slot : 0;
    const int k = live ? sph_pairs_of<false>(c, s, start, skey, dims, a, nullptr, 0) : 0;
    const int lane = threadIdx.x & 31;
    int incl = k;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(cnt + j, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!nb || !live) return;
    const int64_t off = (int64_t)base + incl - k;
    const int64_t room = cap - off;
    int *out = nb + (int64_t)j * cap + off;
    sph_pairs_of<true>(c, s, start, skey, dims, a, out, room > 0 ? room : 0);
    oc[(int64_t)j * n + s.irow(FI_TAG)[a]] = make_int2((int)off, room >= k ? k : 0);
}


/* ------------------------------------------------------------------------ */
/* DEM step VJP */

/* per particle: adjoint of f1 and the wall terms */
__global__ void k_vjp_particles(DevCfg c, int64_t n, double dt, const double *s0, const double *s1,
                                const double *mass, const double *rad, const double *adj, double *fbar,
                                double *racc, double *vmacc, double *grads) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double gk = 0.0, gg = 0.0;
    if (i < n) {
        const double *a = adj + i * ADJ_NC;
        double F[3] = {0, 0, 0}, ra[3] = {0, 0, 0}, va[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) {
            F[d] = a[9 + d] + dt * (a[3 + d] + a[6 + d]); /* f1 feeds f, v1 and vh1 */
            fbar[i * 3 + d] = F[d];
            ra[d] = a[d];
        }
        const double *x1 = s1 + i * ADJ_NC, *x0 = s0 + i * ADJ_NC;
        const double m = mass[i], R = rad[i];
        for (int w = 0; w < (R < 0.0 ? 0 : c.n_walls); w++) {
            double dist = 0.0, vn = 0.0, fn = 0.0;
            for (int d = 0; d < c.nd; d++) {
                const double vhm = x0[6 + d] + 0.5 * dt * x0[9 + d];
                dist += (x1[d] - c.wall_p[w][d]) * c.wall_n[w][d];
                vn += vhm * c.wall_n[w][d];
                fn += F[d] * c.wall_n[w][d];
            }
            const double overlap = R - dist;
            if (!(overlap > 0.0)) continue;
            const double q = fn / m;
            for (int d = 0; d < c.nd; d++) {
                ra[d] += -c.dem_k * c.wall_n[w][d] * q;
                va[d] += -c.dem_gamma * c.wall_n[w][d] * q;
            }
            gk += overlap * q;
            gg += -vn * q;
        }
        for (int d = 0; d < 3; d++) {
            racc[i * 3 + d] = ra[d];
            vmacc[i * 3 + d] = va[d];
        }
    }
    gk = warp_sum_d(gk);
    gg = warp_sum_d(gg);
    if ((threadIdx.x & 31) == 0 && (gk != 0.0 || gg != 0.0)) {
        atomicAdd(&grads[0], gk);
        atomicAdd(&grads[1], gg);
    }
}

/* per contact pair (a, b): the VJP of f_a = s n / m_a */
__global__ void k_vjp_contacts(DevCfg c, const int4 *pairs, const int *cnt, int cap, double dt, const double *s0,
                               const double *s1, const double *mass, const double *rad, const double *fbar,
                               double *racc, double *vmacc, double *grads) {
    const int np = min(*cnt, cap);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double gk = 0.0, gg = 0.0;
    if (q < np) {
        const int4 pr = pairs[q];
        const int a = pr.x, b = pr.y;
        const int sh[3] = {(pr.z & 3) - 1, ((pr.z >> 2) & 3) - 1, ((pr.z >> 4) & 3) - 1};
        double u[3] = {0, 0, 0}, w[3] = {0, 0, 0}, F[3] = {0, 0, 0};
        double r2 = 0.0;
        for (int d = 0; d < c.nd; d++) {
            u[d] = s1[(int64_t)a * ADJ_NC + d] - image_pos(s1[(int64_t)b * ADJ_NC + d], sh[d], c.rmin[d], c.rmax[d]);
            const double vha = s0[(int64_t)a * ADJ_NC + 6 + d] + 0.5 * dt * s0[(int64_t)a * ADJ_NC + 9 + d];
            const double vhb = s0[(int64_t)b * ADJ_NC + 6 + d] + 0.5 * dt * s0[(int64_t)b * ADJ_NC + 9 + d];
            w[d] = vha - vhb;
            F[d] = fbar[(int64_t)a * 3 + d];
            r2 += u[d] * u[d];
        }
        const double r = sqrt(r2), m = mass[a];
        double nn[3] = {0, 0, 0}, wn = 0.0, Fn = 0.0;
        for (int d = 0; d < c.nd; d++) {
            nn[d] = u[d] / r;
            wn += w[d] * nn[d];
            Fn += F[d] * nn[d];
        }
        const double delta = (rad[a] + rad[b]) - r;
        const double s = c.dem_k * delta - c.dem_gamma * wn;
        double ub[3] = {0, 0, 0}, wb[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) {
            const double dsdu = -c.dem_k * nn[d] - (c.dem_gamma / r) * (w[d] - wn * nn[d]);
            ub[d] = (dsdu * Fn + (s / r) * (F[d] - nn[d] * Fn)) / m;
            wb[d] = -c.dem_gamma * nn[d] * Fn / m;
        }
        for (int d = 0; d < c.nd; d++) {
            atomicAdd(&racc[(int64_t)a * 3 + d], ub[d]);
            atomicAdd(&racc[(int64_t)b * 3 + d], -ub[d]);
            atomicAdd(&vmacc[(int64_t)a * 3 + d], wb[d]);
            atomicAdd(&vmacc[(int64_t)b * 3 + d], -wb[d]);
        }
        gk = delta * Fn / m;
        gg = -wn * Fn / m;
    }
    gk = warp_sum_d(gk);
    gg = warp_sum_d(gg);
    if ((threadIdx.x & 31) == 0 && (gk != 0.0 || gg != 0.0)) {
        atomicAdd(&grads[0], gk);
        atomicAdd(&grads[1], gg);
    }
}

/* assemble the adjoint of the state before the step */
__global__ void k_vjp_assemble(int64_t n, double dt, double *adj, const double *racc, const double *vmacc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double *a = adj + i * ADJ_NC;
    for (int d = 0; d < 3; d++) {
        const double rb = racc[i * 3 + d];      /* total adjoint of r1 */
        const double vm = vmacc[i * 3 + d];     /* adjoint of vhm */
        a[d] = rb;                              /* r1 = r0 + dt vh0 */
        a[6 + d] = a[6 + d] + vm + dt * rb;     /* vh1 = vh0 + dt f1, vhm = vh0 + dt/2 f0 */
        a[9 + d] = 0.5 * dt * vm;               /* f0 enters only through vhm */
        /* v0: v1 = v0 + dt f1, nothing else reads v */
    }
}

/* ------------------------------------------------------------------------ */
/* SPH step VJP */

/* VJP of the force of the ordered pair (x, y) on x,
 *   T = [m_y Pi - m_y (pdr2_x + pdr2_y)] G(r) d,  d = r_x - r_y, w = vh_x - vh_y,
 * against the adjoint Fb of f_x.  Adds sign * dT/dd^T Fb to Db and
 * sign * dT/dw^T Fb to Wb (sign -1 when the caller is y), and the adjoints of
 * rho_x (= that of rho_y) to Rb, of pdr2_x (= pdr2_y) to Qb, of alpha to Ab. */
__device__ __forceinline__ void force_pair_vjp(const DevCfg &c, const double *d, const double *w, double r,
                                               double G, double Gp, const double *Fb, double my, double rhox,
                                               double rhoy, double pdr2x, double pdr2y, double sign, double *Db,
                                               double *Wb, double &Rb, double &Qb, double &Ab) {
    double P = 0.0, vdr = 0.0;
    for (int k = 0; k < c.nd; k++) {
        P += Fb[k] * d[k];
        vdr += d[k] * w[k];
    }
    const double ir = 1.0 / r;
    double s = -my * (pdr2x + pdr2y);
    Qb += -my * G * P;
    double coefw = 0.0, coefd = 0.0;
    if (vdr < 0.0) {
        const double viss = vdr * ir, rs = 1.0 / (rhox + rhoy);
        const double Pi = c.alpha_art * viss * (2.0 * c.spsound - 4.0 * viss) * rs;
        const double dPi = c.alpha_art * (2.0 * c.spsound - 8.0 * viss) * rs;
        const double K = G * P;
        s += my * Pi;
        coefw = my * K * dPi * ir;                 /* d viss / d w = d / r */
        coefd = -my * K * dPi * viss * ir * ir;    /* d viss / d d = w / r - viss d / r^2 */
        Rb += -my * K * Pi * rs;
        Ab += my * K * viss * (2.0 * c.spsound - 4.0 * viss) * rs;
        for (int k = 0; k < c.nd; k++) Wb[k] += sign * coefw * d[k];
    }
    const double gpd = Gp * P * ir;
    for (int k = 0; k < c.nd; k++) Db[k] += sign * (s * (G * Fb[k] + gpd * d[k]) + coefw * w[k] + coefd * d[k]);
}

/* tag-order intermediates of the step from its start state s0 */
__global__ void k_sadj_pre(DevCfg c, int64_t n, double dt, const double *s0, const int *typ, double *aux) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *x = s0 + i * ADJ_NC;
    double *o = aux + i * ADJ_AUX;
    const double hd = 0.5 * dt;
    const bool sph = typ[i] == T_SPH;
    for (int d = 0; d < 3; d++) {
        o[d] = x[d] + hd * x[6 + d];
        o[3 + d] = sph ? x[6 + d] + hd * x[9 + d] : x[6 + d];
    }
    const double rho = x[12] + hd * x[13];
    const double q = rho / c.refd, q2 = q * q;
    o[6] = rho;
    o[7] = c.prb * (q2 * q2 * q2 * q - 1.0) / (rho * rho);
}

/* continuity (end phase, pairs at r1): adjoints of r1 and vh1, then of f1 */
__global__ void k_sadj_end(DevCfg c, int64_t n, double dt, const double *s1, const double *mass, const double *hh,
                           const int *typ, const int *nb, const int2 *oc, const double *adj, double *racc,
                           double *vh1b, double *fbar) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double hd = 0.5 * dt;
    const double *xa = s1 + a * ADJ_NC, *aa = adj + a * ADJ_NC;
    const double Da = aa[13] + hd * aa[12], ma = mass[a], ha = hh[a];
    double rb[3] = {0, 0, 0}, wb[3] = {0, 0, 0};
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        const int e = nb[o.x + k];
        const int b = e & ((1 << SH_SHIFT) - 1);
        const int code = (int)((unsigned)e >> SH_SHIFT);
        const int sh[3] = {(code & 3) - 1, ((code >> 2) & 3) - 1, ((code >> 4) & 3) - 1};
        const double *xb = s1 + (int64_t)b * ADJ_NC, *ab = adj + (int64_t)b * ADJ_NC;
        double d[3] = {0, 0, 0}, w[3] = {0, 0, 0}, r2 = 0.0, wd = 0.0;
        for (int q = 0; q < c.nd; q++) {
            d[q] = xa[q] - image_pos(xb[q], sh[q], c.rmin[q], c.rmax[q]);
            w[q] = xa[6 + q] - xb[6 + q];
            r2 += d[q] * d[q];
            wd += w[q] * d[q];
        }
        const double r = sqrt(r2);
        if (!(r > 0.0)) continue;
        double G, Gp;
        grad_factor(c, r, ha, hh[b], G, Gp);
        /* own term m_b D_a and the partner's m_a D_b: d and w flip sign together */
        const double coef = mass[b] * Da + ma * (ab[13] + hd * ab[12]);
        for (int q = 0; q < c.nd; q++) {
            rb[q] += coef * (G * w[q] + Gp * wd * d[q] / r);
            wb[q] += coef * G * d[q];
        }
    }
    const bool sph = typ[a] == T_SPH;
    for (int q = 0; q < 3; q++) {
        const double rt = aa[q] + rb[q];                 /* r1 = r_s + hd vh1 */
        const double vt = aa[6 + q] + wb[q] + hd * rt;   /* total adjoint of vh1 */
        racc[a * 3 + q] = rt;
        vh1b[a * 3 + q] = vt;
        fbar[a * 3 + q] = sph ? aa[9 + q] + dt * (vt + aa[3 + q]) : 0.0;  /* f1 feeds f, vh1, v1 */
    }
}

/* force (middle phase, pairs at r_s), EOS, and the adjoint of the state
 * before the step */
__global__ void k_sadj_mid(DevCfg c, int64_t n, double dt, const double *aux, const double *mass, const double *hh,
                           const int *typ, const int *nb, const int2 *oc, const double *fbar, const double *racc,
                           const double *vh1b, double *adj, double *grads) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double Ab = 0.0;
    if (a < n) {
        const double hd = 0.5 * dt;
        const double *xa = aux + a * ADJ_AUX;
        const double ma = mass[a], ha = hh[a];
        const bool sph_a = typ[a] == T_SPH;
        double Fa[3] = {0, 0, 0};
        for (int q = 0; q < c.nd; q++) Fa[q] = fbar[a * 3 + q];
        double Db[3] = {0, 0, 0}, Wb[3] = {0, 0, 0}, Rb = 0.0, Qb = 0.0, Adum = 0.0;
        const int2 o = oc[a];
        for (int k = 0; k < o.y; k++) {
            const int e = nb[o.x + k];
            const int b = e & ((1 << SH_SHIFT) - 1);
            const int code = (int)((unsigned)e >> SH_SHIFT);
            const int sh[3] = {(code & 3) - 1, ((code >> 2) & 3) - 1, ((code >> 4) & 3) - 1};
            const double *xb = aux + (int64_t)b * ADJ_AUX;
            double d[3] = {0, 0, 0}, w[3] = {0, 0, 0}, md[3] = {0, 0, 0}, mw[3] = {0, 0, 0}, r2 = 0.0;
            for (int q = 0; q < c.nd; q++) {
                d[q] = xa[q] - image_pos(xb[q], sh[q], c.rmin[q], c.rmax[q]);
                w[q] = xa[3 + q] - xb[3 + q];
                md[q] = -d[q];
                mw[q] = -w[q];
                r2 += d[q] * d[q];
            }
            const double r = sqrt(r2);
            if (!(r > 0.0)) continue;
            double G, Gp;
            grad_factor(c, r, ha, hh[b], G, Gp);
            /* a's own pair (a, b); an SPHB particle's force is read by nothing */
            if (sph_a)
                force_pair_vjp(c, d, w, r, G, Gp, Fa, mass[b], xa[6], xb[6], xa[7], xb[7], 1.0, Db, Wb, Rb, Qb, Ab);
            /* the partner's pair (b, a): r_a and vh_a enter it with a minus sign */
            if (typ[b] == T_SPH) {
                double Fbv[3] = {0, 0, 0};
                for (int q = 0; q < c.nd; q++) Fbv[q] = fbar[(int64_t)b * 3 + q];
                force_pair_vjp(c, md, mw, r, G, Gp, Fbv, ma, xb[6], xa[6], xb[7], xa[7], -1.0, Db, Wb, Rb, Qb, Adum);
            }
        }
        /* EOS: d pdr2 / d rho = PRB (5 x^7 + 2) / rho^3, x = rho / refd */
        const double rho = xa[6], x = rho / c.refd, x2 = x * x;
        const double dpdr2 = c.prb * (5.0 * (x2 * x2 * x2 * x) + 2.0) / (rho * rho * rho);
        double *aa = adj + a * ADJ_NC;
        const double rhos_b = aa[12] + Rb + Qb * dpdr2;    /* rho1 = rho_s + ..., force, EOS */
        for (int q = 0; q < 3; q++) {
            const double rs_b = racc[a * 3 + q] + Db[q];    /* total adjoint of r_s */
            aa[q] = rs_b;                                    /* r_s = r0 + hd vh0 */
            aa[6 + q] = vh1b[a * 3 + q] + Wb[q] + hd * rs_b; /* vh1 = vh0 + dt f1, vh_s, r_s */
            aa[9 + q] = sph_a ? hd * Wb[q] : 0.0;            /* vh_s = vh0 + hd f0 */
            /* v0: v1 = v0 + dt f1 only */
        }
        aa[12] = rhos_b;            /* rho_s = rho0 + hd dddt0 */
        aa[13] = hd * rhos_b;
    }
    Ab = warp_sum_d(Ab);
    if ((threadIdx.x & 31) == 0 && Ab != 0.0) atomicAdd(&grads[2], Ab);
}

/* ------------------------------------------------------------------------ */
/* SPH step VJP, mixed precision: the same formulas with FP32 pair math.
 * Positions enter as double-float pairs (hi = (float)r, lo = (float)(r - hi)),
 * so a pair's displacement (hi_a - hi_b) + (lo_a - lo_b) keeps ~1e-7 of
 * itself without FP64 work per pair; velocities, densities, pdr2 and the
 * adjoints are FP32; per-particle sums are Kahan-compensated and land in the
 * FP64 adjoint state once.
 *
 * Records (tag order), middle state:  M0 = (r_s hi, 1/h), M1 = (r_s lo, m),
 * M2 = (vh_s, rho_s), M3 = (adjoint of f1, pdr2_s); end state: E0 = (r1 hi,
 * 1/h), E1 = (r1 lo, m), E2 = (vh1, adjoint of dddt1 + hd adjoint of rho1). */
enum { R_M0 = 0, R_M1, R_M2, R_M3, R_E0, R_E1, R_E2 };

template <int ND>
__device__ __forceinline__ void force_pair_vjp32(float alpha, float c0, const float *d, const float *w, float r,
                                                 float G, float Gp, const float *Fb, float my, float rhox, float rhoy,
                                                 float pdr2x, float pdr2y, float sign, Kf *Db, Kf *Wb, Kf &Rb,
                                                 Kf &Qb, float &Ab) {
    float P = 0.f, vdr = 0.f;
#pragma unroll
    for (int k = 0; k < ND; k++) {
        P = fmaf(Fb[k], d[k], P);
        vdr = fmaf(d[k], w[k], vdr);
    }
    const float ir = 1.f / r;
    float s = -my * (pdr2x + pdr2y);
    Qb.add(-my * G * P);
    float coefw = 0.f, coefd = 0.f;
    if (vdr < 0.f) {
        const float viss = vdr * ir, rs = 1.f / (rhox + rhoy);
        const float Pi = alpha * viss * (2.f * c0 - 4.f * viss) * rs;
        const float dPi = alpha * (2.f * c0 - 8.f * viss) * rs;
        const float K = G * P;
        s += my * Pi;
        coefw = my * K * dPi * ir;
        coefd = -my * K * dPi * viss * ir * ir;
        Rb.add(-my * K * Pi * rs);
        Ab += my * K * viss * (2.f * c0 - 4.f * viss) * rs;
#pragma unroll
        for (int k = 0; k < ND; k++) Wb[k].add(sign * coefw * d[k]);
    }
    const float gpd = Gp * P * ir;
#pragma unroll
    for (int k = 0; k < ND; k++) Db[k].add(sign * (s * (G * Fb[k] + gpd * d[k]) + coefw * w[k] + coefd * d[k]));
}

/* decode a table entry: partner tag and the image displacement to add */
template <int ND>
__device__ __forceinline__ int entry_of(const DevCfg &c, int e, float *img) {
    const int code = (int)((unsigned)e >> SH_SHIFT);
#pragma unroll
    for (int q = 0; q < ND; q++) {
        const int sh = ((code >> (2 * q)) & 3) - 1;
        img[q] = sh == 0 ? 0.f : (float)(sh * (c.rmax[q] - c.rmin[q]));
    }
    return e & ((1 << SH_SHIFT) - 1);
}

/* the FP32 records of one step from its FP64 start / end states */
__global__ void k_sadj_pre32(DevCfg c, int64_t n, double dt, const double *s0, const double *s1, const double *adj,
                             const double *mass, const double *hh, const int *typ, float4 *rec) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *x0 = s0 + i * ADJ_NC, *x1 = s1 + i * ADJ_NC, *aa = adj + i * ADJ_NC;
    const double hd = 0.5 * dt;
    const bool sph = typ[i] == T_SPH;
    const float ih = (float)(1.0 / hh[i]), m = (float)mass[i];
    float hi[3], lo[3], vh[3];
    for (int d = 0; d < 3; d++) {
        split2(x0[d] + hd * x0[6 + d], hi[d], lo[d]);
        vh[d] = (float)(sph ? x0[6 + d] + hd * x0[9 + d] : x0[6 + d]);
    }
    const double rho = x0[12] + hd * x0[13];
    const double q = rho / c.refd, q2 = q * q;
    const double pdr2 = c.prb * (q2 * q2 * q2 * q - 1.0) / (rho * rho);
    rec[R_M0 * n + i] = make_float4(hi[0], hi[1], hi[2], ih);
    rec[R_M1 * n + i] = make_float4(lo[0], lo[1], lo[2], m);
    rec[R_M2 * n + i] = make_float4(vh[0], vh[1], vh[2], (float)rho);
    rec[R_M3 * n + i] = make_float4(0.f, 0.f, 0.f, (float)pdr2);
    for (int d = 0; d < 3; d++) split2(x1[d], hi[d], lo[d]);
    rec[R_E0 * n + i] = make_float4(hi[0], hi[1], hi[2], ih);
    rec[R_E1 * n + i] = make_float4(lo[0], lo[1], lo[2], m);
    rec[R_E2 * n + i] = make_float4((float)x1[6], (float)x1[7], (float)x1[8], (float)(aa[13] + hd * aa[12]));
}

template <int ND>
__global__ void __launch_bounds__(128) k_sadj_end32(DevCfg c, int64_t n, double dt, const int *typ,
                                                    const int *__restrict__ nb, const int2 *__restrict__ oc,
                                                    const double *adj, double *racc, double *vh1b, float4 *rec) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const float4 *E0 = rec + R_E0 * n, *E1 = rec + R_E1 * n, *E2 = rec + R_E2 * n;
    const float wcon = (float)c.wcon;
    const float4 p0 = E0[a], p1 = E1[a], p2 = E2[a];
    const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
    Kf rb[ND], wb[ND];
    const int2 o = oc[a];
    for (int k = 0; k < o.y; k++) {
        float img[3];
        const int b = entry_of<ND>(c, __ldg(nb + o.x + k), img);
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
        const float coef = q1.w * p2.w + p1.w * q2.w;  /* m_b D_a + m_a D_b */
        const float gw = Gp * wd / r;
#pragma unroll
        for (int q = 0; q < ND; q++) {
            rb[q].add(coef * (G * w[q] + gw * d[q]));
            wb[q].add(coef * G * d[q]);
        }
    }
    const double hd = 0.5 * dt;
    const double *aa = adj + a * ADJ_NC;
    const bool sph = typ[a] == T_SPH;
    float F[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < 3; q++) {
        const double rt = aa[q] + (q < ND ? rb[q].value() : 0.0);
        const double vt = aa[6 + q] + (q < ND ? wb[q].value() : 0.0) + hd * rt;
        racc[a * 3 + q] = rt;
        vh1b[a * 3 + q] = vt;
        F[q] = sph ? (float)(aa[9 + q] + dt * (vt + aa[3 + q])) : 0.f;
    }
    float4 *M3 = rec + R_M3 * n;
    M3[a] = make_float4(F[0], F[1], F[2], M3[a].w);
}

template <int ND>
__global__ void __launch_bounds__(128) k_sadj_mid32(DevCfg c, int64_t n, double dt, const double *s0,
                                                    const int *typ, const int *__restrict__ nb,
                                                    const int2 *__restrict__ oc, const double *racc,
                                                    const double *vh1b, const float4 *__restrict__ rec, double *adj,
                                                    double *grads) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float Ab = 0.f;
    if (a < n) {
        const float4 *M0 = rec + R_M0 * n, *M1 = rec + R_M1 * n, *M2 = rec + R_M2 * n, *M3 = rec + R_M3 * n;
        const float wcon = (float)c.wcon, alpha = (float)c.alpha_art, c0 = (float)c.spsound;
        const float4 p0 = M0[a], p1 = M1[a], p2 = M2[a], p3 = M3[a];
        const float pa[3] = {p0.x, p0.y, p0.z}, la[3] = {p1.x, p1.y, p1.z}, va[3] = {p2.x, p2.y, p2.z};
        const float Fa[3] = {p3.x, p3.y, p3.z};
        const bool own = Fa[0] != 0.f || Fa[1] != 0.f || Fa[2] != 0.f;
        Kf Db[ND], Wb[ND], Rb, Qb;
        float Adum = 0.f;
        const int2 o = oc[a];
        for (int k = 0; k < o.y; k++) {
            float img[3];
            const int b = entry_of<ND>(c, __ldg(nb + o.x + k), img);
            const float4 q0 = M0[b], q1 = M1[b], q2 = M2[b], q3 = M3[b];
            const float pb[3] = {q0.x, q0.y, q0.z}, lb[3] = {q1.x, q1.y, q1.z}, vb[3] = {q2.x, q2.y, q2.z};
            const float Fb[3] = {q3.x, q3.y, q3.z};
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
            if (own)
                force_pair_vjp32<ND>(alpha, c0, d, w, r, G, Gp, Fa, q1.w, p2.w, q2.w, p3.w, q3.w, 1.f, Db, Wb, Rb, Qb,
                                     Ab);
            if (Fb[0] != 0.f || Fb[1] != 0.f || Fb[2] != 0.f)
                force_pair_vjp32<ND>(alpha, c0, md, mw, r, G, Gp, Fb, p1.w, q2.w, p2.w, q3.w, p3.w, -1.f, Db, Wb, Rb,
                                     Qb, Adum);
        }
        const double hd = 0.5 * dt;
        const double *x0 = s0 + a * ADJ_NC;
        const double rho = x0[12] + hd * x0[13], x = rho / c.refd, x2 = x * x;
        const double dpdr2 = c.prb * (5.0 * (x2 * x2 * x2 * x) + 2.0) / (rho * rho * rho);
        double *aa = adj + a * ADJ_NC;
        const double rhos_b = aa[12] + Rb.value() + Qb.value() * dpdr2;
        const bool sph_a = typ[a] == T_SPH;
        for (int q = 0; q < 3; q++) {
            const double D = q < ND ? Db[q].value() : 0.0, W = q < ND ? Wb[q].value() : 0.0;
            const double rs_b = racc[a * 3 + q] + D;
            aa[q] = rs_b;
            aa[6 + q] = vh1b[a * 3 + q] + W + hd * rs_b;
            aa[9 + q] = sph_a ? hd * W : 0.0;
        }
        aa[12] = rhos_b;
        aa[13] = hd * rhos_b;
    }
    Ab += __shfl_xor_sync(0xffffffffu, Ab, 16);
    Ab += __shfl_xor_sync(0xffffffffu, Ab, 8);
    Ab += __shfl_xor_sync(0xffffffffu, Ab, 4);
    Ab += __shfl_xor_sync(0xffffffffu, Ab, 2);
    Ab += __shfl_xor_sync(0xffffffffu, Ab, 1);
    if ((threadIdx.x & 31) == 0 && Ab != 0.f) atomicAdd(&grads[2], (double)Ab);
}

void save_state(sphdem_ctx *c, double *dst, const int *slot = nullptr, int K = 1) {
    k_save<<<grid_for(c->n, ABLK), ABLK, 0, c->stream>>>(c->A, c->n, dst, slot, K);
}

void restore_state(sphdem_ctx *c, const double *src, const DevGlobals &g) {
    k_restore<<<grid_for(c->n, ABLK), ABLK, 0, c->stream>>>(c->A, c->n, src);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(c->g, &g, sizeof(g), cudaMemcpyHostToDevice, c->stream));
}

DevGlobals read_globals(sphdem_ctx *c) {
    DevGlobals g;
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(&g, c->g, sizeof(g), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return g;
}

int one_step(sphdem_ctx *c) {
    const int rc = sphdem_step(c, 1);
    if (rc) throw std::string("step: ") + c->err;
    return rc;
}

void sph_pairs(sphdem_ctx *c, int *nb, int2 *oc, int *cnt, const int *slot) {
    AdjointData *a = c->adj;
    k_sph_pairs<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->buf.skey, c->g, c->n, nb,
                                                            oc, cnt, a->pair_cap, slot);
}

/* One replayed fluid or coupled step with its taps, as a CUDA graph (one per
 * buffer parity): the phases of the step, the middle pairs after the middle
 * rebuild (coupled: also the fluid -> DEM pairs and the positions), the end
 * pairs after the end rebuild (coupled: also the FPI and contact pairs), the
 * state after the step (all at the segment slot a->slot), then slot += 1. */
void replay_sph_step(sphdem_ctx *c) {
    AdjointData *a = c->adj;
    cudaGraphExec_t &ge = a->graph[c->flipped ? 1 : 0];
    if (!ge) {
        cudaGraph_t graph = nullptr;
        const bool p0 = c->flipped;
        c->in_capture = true;
        SPHDEM_CUDA_CHECK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        /* mixed coupled handles: the forward coupling passes write the pair tables */
        if (a->mode == ADJ_MODE_COUPLED) c->tap = cpl_forward_taps(c, a);
        try {
            for (int p = SPHDEM_HOOK_BEFORE_START; p <= SPHDEM_HOOK_AFTER_END; p++) {
                phase_sequence(c, p);
                const bool mixed = c->cfg.precision == SPHDEM_PREC_MIXED && c->mx_maxn > 0;
                if (p == SPHDEM_PHASE_MIDDLE) {
                    if (mixed) mixed_adj_pairs(c, a->nb_mid, a->oc_mid, a->pair_cnt, a->pair_cap, a->slot);
                    else sph_pairs(c, a->nb_mid, a->oc_mid, a->pair_cnt, a->slot);
                    if (a->mode == ADJ_MODE_COUPLED) cpl_taps_middle(c, a);
                }
                if (p == SPHDEM_PHASE_END) {
                    if (mixed) mixed_adj_pairs(c, a->nb_end, a->oc_end, a->cnt_end, a->pair_cap, a->slot);
                    else sph_pairs(c, a->nb_end, a->oc_end, a->cnt_end, a->slot);
                    if (a->mode == ADJ_MODE_COUPLED) cpl_taps_end(c, a);
                }
            }
            save_state(c, a->seg, a->slot, a->K);
            k_slot_inc<<<1, 32, 0, c->stream>>>(a->slot);
        } catch (...) {
            c->in_capture = false;
            c->tap = nullptr;
            cudaStreamEndCapture(c->stream, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        c->in_capture = false;
        c->tap = nullptr;
        SPHDEM_CUDA_CHECK(cudaStreamEndCapture(c->stream, &graph));
        if (c->flipped != p0) {
            cudaGraphDestroy(graph);
            throw std::string("a step must rebuild an even number of times");
        }
        const cudaError_t e = cudaGraphInstantiate(&ge, graph, 0);
        cudaGraphDestroy(graph);
        SPHDEM_CUDA_CHECK(e);
    }
    SPHDEM_CUDA_CHECK(cudaGraphLaunch(ge, c->stream));
}

/* the steps of a segment with their taps (the states after each step, the
 * contacts / pair tables of each step), from the segment's first state */
void replay_dem(sphdem_ctx *c, AdjointData *a, int steps, int cap) {
    const int64_t n = c->n;
    for (int j = 1; j <= steps; j++) {
        one_step(c);
        save_state(c, a->seg + (size_t)j * n * ADJ_NC);
        k_contacts<<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->buf.skey, c->g, n,
                                                            a->pairs + (size_t)(j - 1) * cap, a->pair_cnt + j - 1,
                                                            cap);
    }
}

void backward_dem(sphdem_ctx *c, AdjointData *a, int steps, double dt, int cap) {
    const int64_t n = c->n;
    for (int j = steps; j >= 1; j--) {
        const double *s0 = a->seg + (size_t)(j - 1) * n * ADJ_NC, *s1 = a->seg + (size_t)j * n * ADJ_NC;
        k_vjp_particles<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(c->cfg, n, dt, s0, s1, a->mass, a->rad, a->adj,
                                                                  a->fbar, a->racc, a->vmacc, a->grads);
        k_vjp_contacts<<<grid_for(cap, ABLK), ABLK, 0, c->stream>>>(
            c->cfg, a->pairs + (size_t)(j - 1) * cap, a->pair_cnt + j - 1, cap, dt, s0, s1, a->mass, a->rad,
            a->fbar, a->racc, a->vmacc, a->grads);
        k_vjp_assemble<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(n, dt, a->adj, a->racc, a->vmacc);
    }
}

/* the steps of a segment with their taps into tape block a->blk */
void replay_sph(sphdem_ctx *c, AdjointData *a, int steps) {
    const int64_t n = c->n;
    const size_t s0 = (size_t)a->blk * a->K;
    k_slot_set<<<1, 32, 0, c->stream>>>(a->slot, (int)s0);
    /* a particle that stops being SPH/SPHB (deleted) keeps an empty list */
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->oc_mid + s0 * n, 0, (size_t)a->K * n * sizeof(int2), c->stream));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->oc_end + s0 * n, 0, (size_t)a->K * n * sizeof(int2), c->stream));
    if (a->mode == ADJ_MODE_COUPLED) cpl_reset_segment(c, a);
    for (int j = 1; j <= steps; j++) replay_sph_step(c);
}

void backward_sph(sphdem_ctx *c, AdjointData *a, int steps, double dt) {
    const int64_t n = c->n, cap = a->pair_cap;
    const size_t sb = (size_t)a->blk * a->K, stb = (size_t)a->blk * (a->K + 1);
    for (int j = steps; j >= 1; j--) {
        const double *s0 = a->seg + (stb + j - 1) * n * ADJ_NC, *s1 = a->seg + (stb + j) * n * ADJ_NC;
        const int *nbm = a->nb_mid + (sb + j - 1) * cap, *nbe = a->nb_end + (sb + j - 1) * cap;
        const int2 *ocm = a->oc_mid + (sb + j - 1) * n, *oce = a->oc_end + (sb + j - 1) * n;
        if (a->rec) {
            k_sadj_pre32<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(c->cfg, n, dt, s0, s1, a->adj, a->mass, a->hh,
                                                                    a->typ, a->rec);
#define L_(ND)                                                                                                  \
    do {                                                                                                        \
        k_sadj_end32<ND><<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, n, dt, a->typ, nbe, oce, a->adj, a->racc, \
                                                                  a->vmacc, a->rec);                             \
        k_sadj_mid32<ND><<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, n, dt, s0, a->typ, nbm, ocm, a->racc,     \
                                                                  a->vmacc, a->rec, a->adj, a->grads);           \
    } while (0)
            if (c->cfg.nd == 3) L_(3);
            else if (c->cfg.nd == 2) L_(2);
            else L_(1);
#undef L_
            continue;
        }
        k_sadj_pre<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(c->cfg, n, dt, s0, a->typ, a->aux);
        k_sadj_end<<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, n, dt, s1, a->mass, a->hh, a->typ, nbe, oce,
                                                            a->adj, a->racc, a->vmacc, a->fbar);
        k_sadj_mid<<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, n, dt, a->aux, a->mass, a->hh, a->typ, nbm, ocm,
                                                            a->fbar, a->racc, a->vmacc, a->adj, a->grads);
    }
}

void backward_cpl(sphdem_ctx *c, AdjointData *a, int steps, double dt) {
    for (int j = steps; j >= 1; j--) cpl_backward_step(c, a, j, dt);
}

/* How many segments' tapes the store holds: the handle's tape memory
 * (sphdem_adjoint_set_tape_memory) over the bytes of one segment's tape,
 * between 1 and the segment count; DEM handles keep one. */
int tape_blocks(sphdem_ctx *c, AdjointData *a, int nseg) {
    if (a->mode == ADJ_MODE_DEM || nseg <= 1 || c->adj_tape_mem == 0) return 1;
    const int64_t n = c->n, K = a->K;
    int64_t blk = (K + 1) * n * ADJ_NC * (int64_t)sizeof(double) + 2 * K * (int64_t)sizeof(int) +
                  K * (2 * a->pair_cap * (int64_t)sizeof(int) + 2 * n * (int64_t)sizeof(int2));
    if (a->mode == ADJ_MODE_COUPLED)
        blk += K * ((a->cpl.cap + a->fpi.cap + a->ct_cap) * (int64_t)sizeof(int) + 3 * n * (int64_t)sizeof(int2) +
                    3 * (int64_t)sizeof(int) + n * RM_NC * (int64_t)sizeof(double));
    int64_t budget = c->adj_tape_mem;
    if (budget < 0) {   /* half of the device memory free now */
        size_t fr = 0, tot = 0;
        SPHDEM_CUDA_CHECK(cudaMemGetInfo(&fr, &tot));
        budget = (int64_t)(fr / 2);
    }
    return (int)std::max<int64_t>(1, std::min<int64_t>(nseg, budget / blk));
}

/* buffers of the tape store (a->nblk blocks of one segment's tape) and of
 * the reverse sweep */
void alloc_backward(sphdem_ctx *c, AdjointData *a) {
    if (a->seg) return;
    const int64_t n = c->n;
    const int K = a->K * a->nblk;   /* step slots of the store */
    const size_t sbytes = (size_t)n * ADJ_NC * sizeof(double);
    const int cap = ADJ_MAX_CONTACTS * (int)n;
    const bool sph = a->mode == ADJ_MODE_SPH, cpl = a->mode == ADJ_MODE_COUPLED;
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->seg, (size_t)(K + a->nblk) * sbytes));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->pair_cnt, (size_t)K * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->adj, sbytes));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->racc, n * 3 * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->vmacc, n * 3 * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->fbar, n * 3 * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->grads, ADJ_NGRAD * sizeof(double)));
    if (sph || cpl) {
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->nb_mid, (size_t)K * a->pair_cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->nb_end, (size_t)K * a->pair_cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->oc_mid, (size_t)K * n * sizeof(int2)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->oc_end, (size_t)K * n * sizeof(int2)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->cnt_end, (size_t)K * sizeof(int)));
        if (cpl)
            cpl_alloc(c, a);
        else if (c->cfg.precision == SPHDEM_PREC_MIXED)
            SPHDEM_CUDA_CHECK(cudaMalloc(&a->rec, (size_t)n * ADJ_NREC * sizeof(float4)));
        else
            SPHDEM_CUDA_CHECK(cudaMalloc(&a->aux, (size_t)n * ADJ_AUX * sizeof(double)));
    } else {
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->pairs, (size_t)K * cap * sizeof(int4)));
    }
}

/* the tape of segment sg into tape block a->blk: from its checkpoint
 * (already the handle's state), the steps with their taps */
void tape_segment(sphdem_ctx *c, AdjointData *a, int sg, int steps) {
    const size_t sbytes = (size_t)c->n * ADJ_NC * sizeof(double);
    const int K = a->K;
    const size_t sb = (size_t)a->blk * K;
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(a->seg + (size_t)a->blk * (K + 1) * c->n * ADJ_NC, a->ckpt[sg], sbytes,
                                      cudaMemcpyDeviceToDevice, c->stream));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->pair_cnt + sb, 0, K * sizeof(int), c->stream));
    if (a->mode == ADJ_MODE_SPH || a->mode == ADJ_MODE_COUPLED) {
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->cnt_end + sb, 0, K * sizeof(int), c->stream));
        replay_sph(c, a, steps);
    } else {
        replay_dem(c, a, steps, ADJ_MAX_CONTACTS * (int)c->n);
    }
}

}  // namespace

std::string adjoint_supported(sphdem_ctx *c, int *mode) {
    const DevCfg &cfg = c->cfg;
    *mode = 0;
    if (!(cfg.flags & SPHDEM_F_FIXED_DT)) return "the adjoint needs a fixed time step";
    if (cfg.flags & SPHDEM_F_CORRECTED_GRADIENT) return "the adjoint does not cover CORRECTED_GRADIENT";
    if (cfg.flags & SPHDEM_F_DEM_BLOCK) return "the adjoint does not cover DEM_BLOCK";
    if (reinit_configured(c->host_cfg)) return "the adjoint does not cover density re-initialisation";
    if (cfg.damptime > 0) return "the adjoint does not cover velocity damping";
    std::vector<int> iam(c->n);
    field_get_int(c, FI_IAM, iam.data());
    bool all_dem = true, all_fluid = true, all_coupled = true;
    for (int t : iam) {
        all_dem = all_dem && (t == T_DEM || t == T_DEAD);
        all_fluid = all_fluid && is_sph_or_sphb(t);
        all_coupled = all_coupled && (is_sph_or_sphb(t) || t == T_DEM);
    }
    if (cfg.liq_dem()) {
        if (cfg.freeze_until >= 0) return "the adjoint does not cover freezing";
        if (all_dem) {
            /* the contact tables hold ADJ_MAX_CONTACTS * n entries, an int */
            if (c->n > INT_MAX / ADJ_MAX_CONTACTS) return "the DEM adjoint covers at most 67,108,863 particles";
            *mode = ADJ_MODE_DEM;
            return "";
        }
        if (!all_coupled)
            return "the coupled adjoint covers SPH, SPH-boundary and DEM particles (no repulsive boundary particles)";
        if (cfg.visc != SPHDEM_VISC_MORRIS) return "the coupled adjoint covers Morris viscosity only";
        if (!(cfg.flags & SPHDEM_F_NO_ANTICLUMPING)) return "the coupled adjoint does not cover anticlumping";
        /* h constant, or following the density under VAR_H_CORRECTION (the
         * sediment3D form; its reverse passes are the FP32 ones) */
        if (cfg.var_h()) {
            if (cfg.flags & SPHDEM_F_CONST_H) return "the coupled adjoint covers VAR_H_CORRECTION with h following density";
            if (cfg.precision != SPHDEM_PREC_MIXED)
                return "the coupled adjoint covers VAR_H_CORRECTION on mixed-precision handles";
        } else if (!(cfg.flags & SPHDEM_F_CONST_H)) {
            return "the coupled adjoint needs a constant smoothing length or VAR_H_CORRECTION";
        }
        if (cfg.gamma != 7.0) return "the coupled adjoint covers the gamma = 7 equation of state";
        if (c->n > (4 << 20)) return "the coupled adjoint covers at most 4M particles";
        *mode = ADJ_MODE_COUPLED;
        return "";
    }
    if (!all_fluid) return "the fluid adjoint covers handles of SPH and SPH-boundary particles only";
    if (cfg.visc != SPHDEM_VISC_ARTIFICIAL) return "the fluid adjoint covers artificial viscosity only";
    if (!(cfg.flags & SPHDEM_F_CONST_H)) return "the fluid adjoint needs a constant smoothing length";
    if (!(cfg.flags & SPHDEM_F_NO_ANTICLUMPING)) return "the fluid adjoint does not cover anticlumping";
    if (cfg.var_h()) return "the fluid adjoint does not cover VAR_H_CORRECTION";
    for (int d = 0; d < cfg.nd; d++)
        if (cfg.periodic[d]) return "the fluid adjoint does not cover periodic axes";
    /* tags fit below the shift code, and int pair counters do not wrap */
    if (c->n > (4 << 20)) return "the fluid adjoint covers at most 4M particles";
    *mode = ADJ_MODE_SPH;
    return "";
}

int adjoint_forward(sphdem_ctx *c, int nsteps, int K, int mode) {
    adjoint_free(c);
    AdjointData *a = new AdjointData;
    c->adj = a;
    a->mode = mode;
    a->nsteps = nsteps;
    a->K = K;
    a->n = c->n;
    const size_t sbytes = (size_t)c->n * ADJ_NC * sizeof(double);
    const int nseg = (nsteps + K - 1) / K;
    for (int s = 0; s <= nseg; s++) {  /* segment starts + the final state */
        double *p = nullptr;
        SPHDEM_CUDA_CHECK(cudaMalloc(&p, sbytes));
        a->ckpt.push_back(p);
    }
    a->ckpt_g.resize(nseg + 1);
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->mass, c->n * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->rad, c->n * sizeof(double)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->typ, c->n * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&a->hh, c->n * sizeof(double)));
    k_save_const<<<grid_for(c->n, ABLK), ABLK, 0, c->stream>>>(c->cfg, c->A, c->n, a->mass, a->rad, a->typ, a->hh);
    if (mode == ADJ_MODE_SPH || mode == ADJ_MODE_COUPLED) {
        /* size the per-step pair lists from the pairs of the current buckets */
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->slot, sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->slot, 0, sizeof(int), c->stream));
        sph_pairs(c, nullptr, nullptr, a->slot, nullptr);
        int n0 = 0;
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(&n0, a->slot, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        a->pair_cap = (int64_t)n0 + n0 / 2 + 4096;
        if (mode == ADJ_MODE_COUPLED) cpl_count_tables(c, a);
    }
    a->nblk = tape_blocks(c, a, nseg);
    for (int s = 0; s < nseg; s++) {
        save_state(c, a->ckpt[s]);
        a->ckpt_g[s] = read_globals(c);
        const int steps = std::min(K, nsteps - s * K);
        if (s >= nseg - a->nblk) {
            /* the backward pass starts with the last segments: record the
             * tapes of those the store holds now instead of replaying them
             * then */
            alloc_backward(c, a);
            a->blk = s - (nseg - a->nblk);
            tape_segment(c, a, s, steps);
            a->taped = 1;
            const int rc = device_status(c);
            if (rc) return rc;
            continue;
        }
        const int rc = sphdem_step(c, steps);
        if (rc) return rc;
    }
    save_state(c, a->ckpt[nseg]);
    a->ckpt_g[nseg] = read_globals(c);
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return SPHDEM_OK;
}

int adjoint_backward(sphdem_ctx *c, const double *seed_r, const double *seed_v, const double *seed_vh,
                     double *grads5, uint32_t *valid, double *dr0, double *dv0, double *dvh0) {
    AdjointData *a = c->adj;
    if (!a || a->n != c->n) throw std::string("no adjoint forward pass recorded for this handle");
    const int64_t n = c->n;
    const int K = a->K;
    const size_t sbytes = (size_t)n * ADJ_NC * sizeof(double);
    const int cap = ADJ_MAX_CONTACTS * (int)n;
    const bool sph = a->mode == ADJ_MODE_SPH, cpl = a->mode == ADJ_MODE_COUPLED;
    alloc_backward(c, a);
    /* seeds: adjoint of the final (r, v, vh) in tag order; f, dens, dddt 0 */
    {
        std::vector<double> h((size_t)n * ADJ_NC, 0.0);
        for (int64_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) {
                h[i * ADJ_NC + d] = seed_r ? seed_r[3 * i + d] : 0.0;
                h[i * ADJ_NC + 3 + d] = seed_v ? seed_v[3 * i + d] : 0.0;
                h[i * ADJ_NC + 6 + d] = seed_vh ? seed_vh[3 * i + d] : 0.0;
            }
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(a->adj, h.data(), sbytes, cudaMemcpyHostToDevice, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->grads, 0, ADJ_NGRAD * sizeof(double), c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    }
    const int nseg = (a->nsteps + K - 1) / K;
    const double dt = a->ckpt_g[0].dt;
    bool overflow = false;
    const int kept0 = a->taped ? nseg - a->nblk : nseg;
    a->taped = 0;   /* block 0 takes the replays below: a later call replays everything */
    for (int sg = nseg - 1; sg >= 0 && !overflow; sg--) {
        const int steps = std::min(K, a->nsteps - sg * K);
        /* the last nblk segments were taped in the forward pass into blocks
         * 0..nblk-1; the earlier ones are replayed into block 0, whose
         * segment the sweep has passed by then */
        if (sg >= kept0) {
            a->blk = sg - kept0;
        } else {
            a->blk = 0;
            restore_state(c, a->ckpt[sg], a->ckpt_g[sg]);
            tape_segment(c, a, sg, steps);
        }
        if (sph || cpl) {
            if (cpl) backward_cpl(c, a, steps, dt);
            else backward_sph(c, a, steps, dt);
        } else {
            backward_dem(c, a, steps, dt, cap);
        }
        SPHDEM_CUDA_CHECK(cudaGetLastError());
        /* list overflow check of this segment */
        std::vector<int> cnt(2 * K, 0);
        const size_t sb = (size_t)a->blk * K;
        SPHDEM_CUDA_CHECK(
            cudaMemcpyAsync(cnt.data(), a->pair_cnt + sb, K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        if (sph || cpl)
            SPHDEM_CUDA_CHECK(
                cudaMemcpyAsync(cnt.data() + K, a->cnt_end + sb, K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        const int64_t lim = (sph || cpl) ? a->pair_cap : cap;
        for (int v : cnt) overflow = overflow || v > lim;
        if (cpl) overflow = overflow || cpl_overflow(c, a);
        const int rc = device_status(c);
        if (rc != SPHDEM_OK) return rc;
    }
    if (overflow) {
        restore_state(c, a->ckpt[nseg], a->ckpt_g[nseg]);
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        return SPHDEM_ERR_CAPACITY;
    }
    /* outputs, then put the handle back at the final state */
    {
        std::vector<double> h((size_t)n * ADJ_NC);
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(h.data(), a->adj, sbytes, cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(
            cudaMemcpyAsync(grads5, a->grads, ADJ_NGRAD * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        for (int64_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) {
                if (dr0) dr0[3 * i + d] = h[i * ADJ_NC + d];
                if (dv0) dv0[3 * i + d] = h[i * ADJ_NC + 3 + d];
                if (dvh0) dvh0[3 * i + d] = h[i * ADJ_NC + 6 + d];
            }
    }
    *valid = SPHDEM_GRAD_POSITIONS;
    if (a->mode == ADJ_MODE_DEM) *valid |= SPHDEM_GRAD_DEM_K | SPHDEM_GRAD_DEM_GAMMA;
    if (sph) *valid |= SPHDEM_GRAD_VISCOSITY;
    if (cpl) *valid |= SPHDEM_GRAD_DEM_K | SPHDEM_GRAD_DEM_GAMMA | SPHDEM_GRAD_VISCOSITY | SPHDEM_GRAD_DRAG_SCALE;
    restore_state(c, a->ckpt[nseg], a->ckpt_g[nseg]);
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return SPHDEM_OK;
}

}  // namespace sphdem
