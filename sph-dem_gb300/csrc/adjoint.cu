/*
 * Adjoint of the DEM step (reverse mode, FP64), with step checkpointing.
 *
 * Scope: handles whose particles are all DEM (LIQ_DEM without fluid: the
 * granular settling configuration), fixed dt, no damping or freezing.  The
 * step the forward path takes for a DEM particle (k_start, k_middle_tail,
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
 *
 * sphdem_adjoint_forward runs the steps through the ordinary path (graph
 * replay) and keeps the state (r, v, vh, f in tag order) and the step
 * globals every `ckpt_every` steps.  sphdem_adjoint_backward walks the
 * segments from the last: it restores the segment's checkpoint into the
 * handle, replays its steps while keeping every step's state and the
 * contact pairs the end phase used (the same exact FP64 predicate and
 * overlap test), then applies the step's vector-Jacobian product in reverse
 * order.  Replays are bit-identical to the first forward pass (the bucket
 * order is a deterministic function of the positions), so the gradients are
 * those of the computed trajectory.  Contacts are scattered with FP64
 * atomics; gamma and k gradients are warp-reduced first.
 */
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"

namespace sphdem {

constexpr int ADJ_NC = 12;         /* r, v, vh, f per particle */
constexpr int ADJ_MAX_CONTACTS = 32;

struct AdjointData {
    int nsteps = 0, K = 0;
    int64_t n = 0;
    std::vector<double *> ckpt;     /* state at steps 0, K, 2K, ... and the final state */
    std::vector<DevGlobals> ckpt_g;
    double *seg = nullptr;          /* (K + 1) states of one segment */
    int4 *pairs = nullptr;          /* contacts of each step of a segment */
    int *pair_cnt = nullptr;        /* K counters */
    double *adj = nullptr;          /* adjoint of the state (ADJ_NC per particle) */
    double *racc = nullptr;         /* accumulated adjoint of r1 through the forces */
    double *vmacc = nullptr;        /* adjoint of vhm */
    double *fbar = nullptr;         /* adjoint of f1 */
    double *mass = nullptr, *rad = nullptr;   /* tag order */
    double *grads = nullptr;        /* d/dk, d/dgamma */
};

void adjoint_free(sphdem_ctx *c) {
    AdjointData *a = c->adj;
    if (!a) return;
    for (double *p : a->ckpt) cudaFree(p);
    cudaFree(a->seg);
    cudaFree(a->pairs);
    cudaFree(a->pair_cnt);
    cudaFree(a->adj);
    cudaFree(a->racc);
    cudaFree(a->vmacc);
    cudaFree(a->fbar);
    cudaFree(a->mass);
    cudaFree(a->rad);
    cudaFree(a->grads);
    delete a;
    c->adj = nullptr;
}

namespace {

constexpr int ABLK = 256;

__global__ void k_save(DevState s, int64_t n, double *dst) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    double *o = dst + (int64_t)s.irow(FI_TAG)[k] * ADJ_NC;
    for (int d = 0; d < 3; d++) {
        o[d] = s.row(FD_R + d)[k];
        o[3 + d] = s.row(FD_V + d)[k];
        o[6 + d] = s.row(FD_VHAT + d)[k];
        o[9 + d] = s.row(FD_F + d)[k];
    }
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
}

__global__ void k_save_const(DevCfg c, DevState s, int64_t n, double *mass, double *rad) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = s.irow(FI_TAG)[k];
    mass[t] = s.row(FD_MASS)[k];
    /* radius, or -1 for a particle that is not (or no longer) DEM */
    rad[t] = s.irow(FI_IAM)[k] != T_DEM ? -1.0 : (s.row(FD_RADIUS)[k] > 0 ? s.row(FD_RADIUS)[k] : c.dem_radius);
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

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

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

void save_state(sphdem_ctx *c, double *dst) {
    k_save<<<grid_for(c->n, ABLK), ABLK, 0, c->stream>>>(c->A, c->n, dst);
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

}  // namespace

std::string adjoint_supported(sphdem_ctx *c) {
    const DevCfg &cfg = c->cfg;
    if (!cfg.liq_dem()) return "the adjoint covers LIQ_DEM handles of DEM particles";
    if (!(cfg.flags & SPHDEM_F_FIXED_DT)) return "the adjoint needs a fixed time step";
    if (cfg.damptime > 0) return "the adjoint does not cover velocity damping";
    if (cfg.freeze_until >= 0) return "the adjoint does not cover freezing";
    std::vector<int> iam(c->n);
    field_get_int(c, FI_IAM, iam.data());
    for (int t : iam)
        if (t != T_DEM && t != T_DEAD) return "the adjoint covers handles whose particles are all DEM";
    return "";
}

int adjoint_forward(sphdem_ctx *c, int nsteps, int K) {
    adjoint_free(c);
    AdjointData *a = new AdjointData;
    c->adj = a;
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
    k_save_const<<<grid_for(c->n, ABLK), ABLK, 0, c->stream>>>(c->cfg, c->A, c->n, a->mass, a->rad);
    for (int s = 0; s < nseg; s++) {
        save_state(c, a->ckpt[s]);
        a->ckpt_g[s] = read_globals(c);
        const int steps = std::min(K, nsteps - s * K);
        const int rc = sphdem_step(c, steps);
        if (rc) return rc;
    }
    save_state(c, a->ckpt[nseg]);
    a->ckpt_g[nseg] = read_globals(c);
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return SPHDEM_OK;
}

int adjoint_backward(sphdem_ctx *c, const double *seed_r, const double *seed_v, const double *seed_vh,
                     double *dk, double *dgamma, double *dr0, double *dv0, double *dvh0) {
    AdjointData *a = c->adj;
    if (!a || a->n != c->n) throw std::string("no adjoint forward pass recorded for this handle");
    const int64_t n = c->n;
    const int K = a->K;
    const size_t sbytes = (size_t)n * ADJ_NC * sizeof(double);
    const int cap = ADJ_MAX_CONTACTS * (int)n;
    if (!a->seg) {
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->seg, (size_t)(K + 1) * sbytes));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->pairs, (size_t)K * cap * sizeof(int4)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->pair_cnt, (size_t)K * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->adj, sbytes));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->racc, n * 3 * sizeof(double)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->vmacc, n * 3 * sizeof(double)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->fbar, n * 3 * sizeof(double)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&a->grads, 2 * sizeof(double)));
    }
    /* seeds: adjoint of the final (r, v, vh, f) in tag order */
    {
        std::vector<double> h((size_t)n * ADJ_NC, 0.0);
        for (int64_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) {
                h[i * ADJ_NC + d] = seed_r ? seed_r[3 * i + d] : 0.0;
                h[i * ADJ_NC + 3 + d] = seed_v ? seed_v[3 * i + d] : 0.0;
                h[i * ADJ_NC + 6 + d] = seed_vh ? seed_vh[3 * i + d] : 0.0;
            }
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(a->adj, h.data(), sbytes, cudaMemcpyHostToDevice, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->grads, 0, 2 * sizeof(double), c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    }
    const int nseg = (a->nsteps + K - 1) / K;
    const double dt = a->ckpt_g[0].dt;
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int steps = std::min(K, a->nsteps - sg * K);
        restore_state(c, a->ckpt[sg], a->ckpt_g[sg]);
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(a->seg, a->ckpt[sg], sbytes, cudaMemcpyDeviceToDevice, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemsetAsync(a->pair_cnt, 0, K * sizeof(int), c->stream));
        for (int j = 1; j <= steps; j++) {
            one_step(c);
            save_state(c, a->seg + (size_t)j * n * ADJ_NC);
            k_contacts<<<grid_for(n, 128), 128, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->buf.skey, c->g, n,
                                                                a->pairs + (size_t)(j - 1) * cap, a->pair_cnt + j - 1,
                                                                cap);
        }
        for (int j = steps; j >= 1; j--) {
            const double *s0 = a->seg + (size_t)(j - 1) * n * ADJ_NC, *s1 = a->seg + (size_t)j * n * ADJ_NC;
            k_vjp_particles<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(c->cfg, n, dt, s0, s1, a->mass, a->rad, a->adj,
                                                                      a->fbar, a->racc, a->vmacc, a->grads);
            k_vjp_contacts<<<grid_for(cap, ABLK), ABLK, 0, c->stream>>>(
                c->cfg, a->pairs + (size_t)(j - 1) * cap, a->pair_cnt + j - 1, cap, dt, s0, s1, a->mass, a->rad,
                a->fbar, a->racc, a->vmacc, a->grads);
            k_vjp_assemble<<<grid_for(n, ABLK), ABLK, 0, c->stream>>>(n, dt, a->adj, a->racc, a->vmacc);
        }
        SPHDEM_CUDA_CHECK(cudaGetLastError());
    }
    /* contact overflow check */
    {
        std::vector<int> cnt(K);
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(cnt.data(), a->pair_cnt, K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        for (int v : cnt)
            if (v > cap) return SPHDEM_ERR_CAPACITY;
    }
    /* outputs, then put the handle back at the final state */
    {
        std::vector<double> h((size_t)n * ADJ_NC);
        double g[2];
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(h.data(), a->adj, sbytes, cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(g, a->grads, sizeof(g), cudaMemcpyDeviceToHost, c->stream));
        SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
        for (int64_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) {
                if (dr0) dr0[3 * i + d] = h[i * ADJ_NC + d];
                if (dv0) dv0[3 * i + d] = h[i * ADJ_NC + 3 + d];
                if (dvh0) dvh0[3 * i + d] = h[i * ADJ_NC + 6 + d];
            }
        *dk = g[0];
        *dgamma = g[1];
    }
    restore_state(c, a->ckpt[nseg], a->ckpt_g[nseg]);
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return SPHDEM_OK;
}

}  // namespace sphdem
