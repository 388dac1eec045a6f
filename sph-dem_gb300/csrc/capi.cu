/*
 * extern "C" entry points of include/sphdem.h.
 *
 * A handle owns: the particle state (two SoA copies in HBM), the bucket
 * arrays, the device-resident step globals, a private CUDA stream and, once
 * a full step has run, a CUDA graph of one step per state parity.  The phase
 * sequence reproduces CsphIncompress::start/middle/end (sphIncompress.cpp:
 * 3-251) with the hooks of run.cpp:112-118 in between.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"

using namespace sphdem;

namespace sphdem {

void launch_begin(sphdem_ctx *c, const char *name) {
    if (!c->timing || c->in_capture) return;
    TimedLaunch t;
    t.name = name;
    cudaEventCreate(&t.ev0);
    cudaEventCreate(&t.ev1);
    cudaEventRecord(t.ev0, c->stream);
    c->launches.push_back(t);
}

void launch_end(sphdem_ctx *c) {
    if (!c->timing || c->in_capture) return;
    cudaEventRecord(c->launches.back().ev1, c->stream);
}

}  // namespace sphdem

namespace {

void collect_times(sphdem_ctx *c) {
    if (c->launches.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto &t : c->launches) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t.ev0, t.ev1);
        auto it = std::find(c->kt_names.begin(), c->kt_names.end(), std::string(t.name));
        size_t k;
        if (it == c->kt_names.end()) {
            c->kt_names.push_back(t.name);
            c->kt_ms.push_back(0.0);
            c->kt_count.push_back(0);
            k = c->kt_names.size() - 1;
        } else {
            k = it - c->kt_names.begin();
        }
        c->kt_ms[k] += ms;
        c->kt_count[k] += 1;
        cudaEventDestroy(t.ev0);
        cudaEventDestroy(t.ev1);
    }
    c->launches.clear();
}

int fail(sphdem_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

/* Read the device error flags (synchronises the stream). */
int check_device(sphdem_ctx *c) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(c, SPHDEM_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, SPHDEM_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    unsigned int err = 0;
    int info = 0;
    cudaMemcpy(&err, &c->g->err, sizeof(err), cudaMemcpyDeviceToHost);
    if (!err) return SPHDEM_OK;
    cudaMemcpy(&info, &c->g->err_info, sizeof(info), cudaMemcpyDeviceToHost);
    for (int code = 1; code < 32; code++)
        if (err & (1u << code)) {
            char buf[256];
            snprintf(buf, sizeof buf, "device reported error %d (info %d): %s", code, info,
                     code == SPHDEM_ERR_CAPACITY ? "bucket grid capacity exceeded or periodic axis too short"
                     : code == SPHDEM_ERR_OUT_OF_RANGE ? "particle outside the bucket grid"
                                                       : "device check failed");
            return fail(c, code, buf);
        }
    return SPHDEM_ERR_CUDA;
}

void build_devcfg(const SphDemConfig &h, DevCfg &c) {
    std::memset(&c, 0, sizeof(c));
    c.nd = h.ndim;
    c.visc = h.visc_model;
    c.precision = h.precision;
    c.flags = h.flags;
    c.n_walls = h.n_walls;
    for (int d = 0; d < 3; d++) {
        c.periodic[d] = d < h.ndim ? h.periodic[d] : 0;
        c.rmin[d] = h.rmin[d];
        c.rmax[d] = h.rmax[d];
        c.dmin[d] = h.domain_min[d];
        c.dmax[d] = h.domain_max[d];
        c.g_sph[d] = h.gravity_sph[d];
        c.g_dem[d] = h.gravity_dem[d];
    }
    c.pi = h.pi;
    c.hfac = h.hfac;
    c.psep = h.psep;
    c.h = h.h;
    c.dens = h.dens;
    c.refd = h.refd;
    c.gamma = h.gamma;
    c.prb = h.prb;
    c.spsound = h.spsound;
    c.viscosity = h.viscosity;
    c.drag_scale = h.drag_scale != 0.0 ? h.drag_scale : 1.0;
    c.alpha_art = h.alpha_artificial;
    c.alpha_mon = h.viscosity * (112.0 / 15.0) / (h.spsound * h.h);  /* viscToAlpha, misc.h:41-43 */
    c.bfac = h.bfac;
    c.maxdt = h.maxdt;
    c.damptime = h.damptime;
    c.dem_radius = h.dem_radius;
    c.dem_dens = h.dem_dens;
    c.dem_k = h.dem_k;
    c.dem_gamma = h.dem_gamma;
    c.dem_sr = h.dem_search_radius;
    c.dem_vol = h.dem_vol;
    c.rc = h.coupling_radius;
    c.dem_timestep = h.dem_timestep;
    c.liq_dem_timestep = h.liq_dem_timestep;
    c.time_drop = h.time_drop_particle;
    c.freeze_until = h.freeze_dem_until;
    for (int w = 0; w < SPHDEM_MAX_WALLS; w++)
        for (int d = 0; d < 3; d++) {
            c.wall_p[w][d] = h.walls[w].point[d];
            c.wall_n[w][d] = h.walls[w].normal[d];
        }
    c.wcon = h.ndim == 2 ? 7.0 / (64.0 * h.pi) : 21.0 / (256.0 * h.pi);
    /* migration test extents */
    for (int d = 0; d < 3; d++) {
        c.dspace[d] = c.dmax[d] - c.dmin[d];
        c.rdspace_f[d] = c.dspace[d] > 0 ? (float)(1.0 / c.dspace[d]) : 0.f;
    }
    /* DEM search grid and the reference DEM bucket map */
    const bool liq = h.flags & SPHDEM_F_LIQ_DEM;
    double cmin = std::max(h.coupling_radius, 2.0 * h.dem_search_radius) * (1.0 + 1e-12);
    if (!(cmin > 0)) cmin = 1.0;
    int ndc = 1;
    for (int d = 0; d < 3; d++) {
        if (d >= h.ndim || !liq) {
            c.ddims[d] = 1;
            c.dcell[d] = 1.0;
            c.dorig[d] = 0.0;
            c.rdcell[d] = 1.0;
            continue;
        }
        const double ext = c.dspace[d];
        if (c.periodic[d]) {
            int m = (int)std::floor(ext / cmin);
            if (m < 3) m = 3;
            c.ddims[d] = m;
            c.dcell[d] = ext / m;
            c.dorig[d] = c.dmin[d];
        } else {
            c.ddims[d] = (int)std::ceil(ext / cmin) + 2;
            c.dcell[d] = cmin;
            c.dorig[d] = c.dmin[d] - cmin;
        }
        c.rdcell[d] = 1.0 / c.dcell[d];
        ndc *= c.ddims[d];
    }
    c.n_dem_cells = liq ? ndc : 0;
    if (liq && h.dem_search_radius > 0) {
        c.dem_cell_off = 2 * h.coupling_radius / h.dem_search_radius - 1;
        c.rdem2_f = (float)(1.0 / (2 * h.dem_search_radius));
        c.couple_num = (int)std::ceil(0.5 * h.coupling_radius / h.dem_search_radius);
        c.couple_lim = std::pow(0.5 * h.coupling_radius / h.dem_search_radius, 2);
        for (int d = 0; d < 3; d++) {
            c.dg_lo[d] = c.dmin[d] + h.coupling_radius;
            double sp = c.dspace[d] - h.coupling_radius;
            sp -= h.coupling_radius;
            c.dg_sp[d] = sp;
            c.dg_rsp_f[d] = sp != 0 ? (float)(1.0 / sp) : 0.f;
        }
    }
    c.two_over_rc = h.coupling_radius > 0 ? 2.0 / h.coupling_radius : 0.0;
    c.rc2 = h.coupling_radius * h.coupling_radius;
    const double hc = h.coupling_radius / 2.0;
    if (hc > 0) {
        c.c_ihn = 1 / std::pow(hc, h.ndim);
        c.c_ihn2 = 1 / std::pow(hc, h.ndim + 2);
        c.c_hinv = 1 / hc;
    }
    c.por_incr = h.ndim == 2 ? (4.0 / 3.0) * h.pi * std::pow(h.dem_radius, 3) / (2.0 * h.dem_radius)
                             : (4.0 / 3.0) * h.pi * std::pow(h.dem_radius, 3);
    {
        const double q = 1.0 / h.hfac;
        const double t = 2.0 - q;
        c.k_anti = q <= 2.0 ? c.wcon * std::pow(t, 4) * (1.0 + 2.0 * q) : 0.0;
    }
    c.f_pi = (float)h.pi;
    c.f_c0 = (float)h.spsound;
    c.f_rpsep = h.psep > 0 ? (float)(1.0 / h.psep) : 0.f;
    c.f_rdelp = h.bfac * h.psep > 0 ? (float)(1.0 / (h.bfac * h.psep)) : 0.f;
}

std::string validate(const SphDemConfig *cfg, const SphDemParticles *p, int64_t cap) {
    if (!cfg || !p) return "null config or particles";
    if (cfg->ndim < 1 || cfg->ndim > 3) return "ndim must be 1, 2 or 3";
    if (p->n <= 0) return "no particles";
    if (cap < p->n) return "capacity smaller than the particle count";
    if (p->n > (int64_t)1 << 26) return "more than 2^26 particles";
    if (!p->iam || !p->r || !p->mass || !p->dens || !p->h) return "iam, r, mass, dens and h are required";
    if (!(cfg->h > 0) || !(cfg->maxdt > 0)) return "h and maxdt must be positive";
    if (cfg->precision != SPHDEM_PREC_FP64 && cfg->precision != SPHDEM_PREC_MIXED) return "unknown precision";
    if (cfg->n_walls < 0 || cfg->n_walls > SPHDEM_MAX_WALLS) return "n_walls out of range";
    for (int d = 0; d < cfg->ndim; d++)
        if (!(cfg->domain_max[d] > cfg->domain_min[d])) return "empty binning domain";
    if (cfg->flags & SPHDEM_F_CORRECTED_GRADIENT) {
        if (cfg->flags & SPHDEM_F_LIQ_DEM) return "CORRECTED_GRADIENT is not combined with LIQ_DEM";
    }
    if (cfg->reinit_dens_every < 0) return "reinit_dens_every must be >= 0";
    if ((cfg->flags & SPHDEM_F_DEM_BLOCK) && !(cfg->flags & SPHDEM_F_LIQ_DEM)) return "DEM_BLOCK needs LIQ_DEM";
    if ((cfg->flags & SPHDEM_F_LIQ_DEM) && !(cfg->dem_search_radius > 0 && cfg->coupling_radius > 0))
        return "LIQ_DEM needs dem_search_radius and coupling_radius";
    if ((cfg->flags & SPHDEM_F_LIQ_DEM) && cfg->precision == SPHDEM_PREC_MIXED) {
        /* the mixed coupling pass packs reference DEM bucket indices (of
         * particles and their periodic images) into 10 bits per axis */
        for (int d = 0; d < cfg->ndim; d++) {
            const double w = 2 * cfg->dem_search_radius;
            const double off = 2 * cfg->coupling_radius / cfg->dem_search_radius - 1;
            const double period = cfg->periodic[d] ? cfg->rmax[d] - cfg->rmin[d] : 0.0;
            const double kmax = (cfg->domain_max[d] - cfg->domain_min[d] + period) / w + off + 2;
            const double kmin = -period / w + off - 2;
            if (kmax > 511 || kmin < -512)
                return "mixed precision: reference DEM bucket indices outside [-512, 511] along an axis";
        }
    }
    for (int64_t i = 0; i < p->n; i++) {
        for (int d = 0; d < 3; d++)
            if (!std::isfinite(p->r[3 * i + d])) return "non-finite position";
        if (!(p->h[i] > 0) || !(p->mass[i] > 0) || !(p->dens[i] > 0)) return "h, mass and dens must be positive";
    }
    return "";
}

void free_ctx(sphdem_ctx *c) {
    if (!c) return;
    adjoint_free(c);
    cudaFree(c->A.d);
    cudaFree(c->A.i);
    cudaFree(c->B.d);
    cudaFree(c->B.i);
    cudaFree(c->g);
    Buffers &b = c->buf;
    cudaFree(b.slot_z);
    for (int *p : {b.skey, b.perm, b.slot, b.slot_tag, b.key, b.cnt, b.start, b.fill, b.bsum, b.fields_d, b.fields_i,
                   b.pair_cnt})
        cudaFree(p);
    cudaFree(c->mx_pos);
    cudaFree(c->mx_vel);
    cudaFree(c->mx_aux);
    cudaFree(c->mx_tg);
    cudaFree(c->mx_om);
    cudaFree(c->mx_nbr);
    cudaFree(c->mx_ncnt);
    cudaFree(c->stage);
    cudaFree(c->mx_q0);
    cudaFree(c->mx_q1);
    cudaFree(c->mx_q2);
    cudaFree(c->mx_dp);
    cudaFree(c->mx_poslo);
    cudaFree(c->mx_rc4);
    cudaFree(c->mx_shep32);
    cudaFree(c->mx_ds);
    cudaFree(c->mx_nb);
    cudaFree(c->mx_win);
    cudaFree(c->mx_bandq);
    cudaFree(c->mx_bandn);
    cudaFree(c->dcfg);
    fields_async_free(c);
    cudaFree(c->cg);
    cudaFree(c->hpred);
    cudaFree(c->delmark);
    for (int k = 0; k < 4; k++)
        if (c->graph[k]) cudaGraphExecDestroy(c->graph[k]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

void run_phase_mixed(sphdem_ctx *c, int phase) {
    const bool liq = c->cfg.liq_dem();
    const bool lists = c->mx_maxn > 0;
    switch (phase) {
        case SPHDEM_PHASE_MIDDLE:
            globals_op(c, OP_MIDDLE_BEGIN);
            rebuild(c);
            mixed::pack(c);
            if (lists) mixed::nlist(c);
            /* calcInvM in FP64 once per rebuild; the pair passes apply it in FP32 */
            if (corrected_gradient(c)) run_invm(c);
            if (liq) {
                mixed::zero_shep(c);
                mixed::porosity(c);
                mixed::dem_drag(c);
            }
            if (lists) {
                /* elementwise EOS; Omega (VAR_H_CORRECTION) is summed inside the force pass */
                mixed::omega_eos(c, false, true);
                mixed::force(c);
            }
            if (liq) run_dem_accel(c);
            globals_op(c, OP_SET_DT);
            run_middle_tail(c);
            break;
        case SPHDEM_PHASE_END:
            run_end_drift(c);
            rebuild(c);
            mixed::pack(c, false);
            if (corrected_gradient(c)) run_invm(c);
            if (lists) {
                mixed::nlist(c);
                mixed::dddt(c);  /* Omega (VAR_H_CORRECTION) is summed inside the continuity pass */
            }
            if (liq) mixed::dem_end(c);
            if (c->host_cfg.flags & SPHDEM_F_DEM_BLOCK) run_dem_block(c);
            run_end_tail(c);
            break;
    }
}

void run_phase(sphdem_ctx *c, int phase) {
    const bool liq = c->cfg.liq_dem();
    /* a DEM-only handle has no FP32 pair pass: its contacts are FP64 on both
     * paths, so the mixed handle runs the FP64 phases */
    if (c->cfg.precision == SPHDEM_PREC_MIXED && !c->mx_dem_only &&
        (phase == SPHDEM_PHASE_MIDDLE || phase == SPHDEM_PHASE_END)) {
        run_phase_mixed(c, phase);
        return;
    }
    switch (phase) {
        case SPHDEM_HOOK_BEFORE_START:
            globals_op(c, OP_STEP_INC);
            c->host_step++;
            break;
        case SPHDEM_PHASE_START:
            run_start(c);
            if (reinit_due(c->host_cfg, c->host_step)) run_reinit_density(c);
            break;
        case SPHDEM_HOOK_BEFORE_MIDDLE:
            run_hook_before_middle(c);
            break;
        case SPHDEM_PHASE_MIDDLE:
            globals_op(c, OP_MIDDLE_BEGIN);
            rebuild(c);
            if (liq) {
                run_porosity(c);
                run_dem_drag(c);
            }
            if (corrected_gradient(c)) run_invm(c);
            run_omega_eos(c, c->cfg.var_h(), true);
            run_force(c);
            if (liq) run_dem_accel(c);
            globals_op(c, OP_SET_DT);
            run_middle_tail(c);
            break;
        case SPHDEM_HOOK_BEFORE_END:
            run_hook_before_end(c);
            break;
        case SPHDEM_PHASE_END:
            run_end_drift(c);
            rebuild(c);
            if (corrected_gradient(c)) run_invm(c);
            if (c->cfg.var_h()) run_omega_eos(c, true, false);
            run_dddt(c);
            if (liq) run_dem_end(c);
            if (c->host_cfg.flags & SPHDEM_F_DEM_BLOCK) run_dem_block(c);
            run_end_tail(c);
            break;
        case SPHDEM_HOOK_AFTER_END:
            run_hook_after_end(c);
            break;
    }
}

void run_full_step(sphdem_ctx *c) {
    for (int p = SPHDEM_HOOK_BEFORE_START; p <= SPHDEM_HOOK_AFTER_END; p++) run_phase(c, p);
}

}  // namespace

namespace sphdem {
void step_sequence(sphdem_ctx *c) { run_full_step(c); }
void phase_sequence(sphdem_ctx *c, int phase) { run_phase(c, phase); }
int device_status(sphdem_ctx *c) { return check_device(c); }
}  // namespace sphdem

extern "C" {

const char *sphdem_version(void) { return "sphdem-gb300 0.1 (sm_103a)"; }

/* text of the calling thread's last failed sphdem_create (no handle exists
 * to hold it) */
static thread_local std::string g_create_err;

int sphdem_last_error(sphdem_handle h, char *buf, size_t len) {
    if (!buf || !len) return SPHDEM_ERR_INVALID;
    const std::string e = h ? h->err : (g_create_err.empty() ? std::string("no handle") : g_create_err);
    std::snprintf(buf, len, "%s", e.c_str());
    return SPHDEM_OK;
}

int sphdem_create(const SphDemConfig *cfg, const SphDemParticles *init, int64_t capacity, sphdem_handle *out) {
    if (!out) return SPHDEM_ERR_INVALID;
    *out = nullptr;
    const std::string v = validate(cfg, init, capacity);
    if (!v.empty()) {
        g_create_err = v;
        fprintf(stderr, "sphdem_create: %s\n", v.c_str());
        return SPHDEM_ERR_INVALID;
    }
    sphdem_ctx *c = new sphdem_ctx();
    try {
        c->host_cfg = *cfg;
        build_devcfg(*cfg, c->cfg);
        c->n = init->n;
        c->cap = capacity;
        SPHDEM_CUDA_CHECK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        for (DevState *s : {&c->A, &c->B}) {
            s->cap = capacity;
            SPHDEM_CUDA_CHECK(cudaMalloc(&s->d, (size_t)NFD * capacity * sizeof(double)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&s->i, (size_t)NFI * capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMemset(s->d, 0, (size_t)NFD * capacity * sizeof(double)));
            SPHDEM_CUDA_CHECK(cudaMemset(s->i, 0, (size_t)NFI * capacity * sizeof(int)));
        }
        /* upload in tag order */
        const int64_t n = c->n;
        std::vector<double> row(n);
        auto up = [&](int f, const std::vector<double> &v) {
            SPHDEM_CUDA_CHECK(cudaMemcpy(c->A.row(f), v.data(), n * sizeof(double), cudaMemcpyHostToDevice));
        };
        auto vec = [&](int base, const double *src, double dflt, const double *fallback) {
            for (int d = 0; d < 3; d++) {
                for (int64_t i = 0; i < n; i++)
                    row[i] = src ? src[3 * i + d] : (fallback ? fallback[3 * i + d] : dflt);
                up(base + d, row);
            }
        };
        auto sca = [&](int f, const double *src, double dflt) {
            for (int64_t i = 0; i < n; i++) row[i] = src ? src[i] : dflt;
            up(f, row);
        };
        vec(FD_R, init->r, 0.0, nullptr);
        vec(FD_V, init->v, 0.0, nullptr);
        vec(FD_VHAT, init->vhat, 0.0, init->v);
        vec(FD_N1, init->norm1, 0.0, nullptr);
        vec(FD_N2, init->norm2, 0.0, nullptr);
        vec(FD_N3, init->norm3, 0.0, nullptr);
        sca(FD_MASS, init->mass, 0.0);
        sca(FD_DENS, init->dens, 0.0);
        sca(FD_H, init->h, 0.0);
        sca(FD_RADIUS, init->radius, 0.0);
        sca(FD_POR, nullptr, 1.0);  /* Cparticle() sets porosity = 1 (particle.h:82) */
        std::vector<int> irow(n);
        for (int64_t i = 0; i < n; i++) irow[i] = init->iam[i];
        SPHDEM_CUDA_CHECK(cudaMemcpy(c->A.irow(FI_IAM), irow.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        for (int64_t i = 0; i < n; i++) irow[i] = (int)i;
        SPHDEM_CUDA_CHECK(cudaMemcpy(c->A.irow(FI_TAG), irow.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        for (int64_t i = 0; i < n; i++) irow[i] = init->concave ? init->concave[i] != 0 : 1;
        SPHDEM_CUDA_CHECK(cudaMemcpy(c->A.irow(FI_CONCAVE), irow.data(), n * sizeof(int), cudaMemcpyHostToDevice));

        /* bucket grid capacity: SPH grid at half the smallest of H and the
         * largest initial h (h may shrink until then), DEM grid fixed */
        double hmax0 = 0;
        for (int64_t i = 0; i < n; i++) hmax0 = std::max(hmax0, init->h[i]);
        const double sr_min = 0.5 * std::min(cfg->h, hmax0);
        long long sc = 1;
        int win_cap = 1; /* bucket indices along any one axis */
        for (int d = 0; d < cfg->ndim; d++) {
            const long long nd = (long long)((cfg->domain_max[d] - cfg->domain_min[d]) / (2.0 * sr_min)) + 9;
            sc *= nd;
            win_cap = (int)std::max<long long>(win_cap, std::min<long long>(nd, 1ll << 30));
        }
        if (sc > (1ll << 30)) throw std::string("bucket grid too large for the domain / smoothing length");
        c->cfg.sph_cells_cap = (int)sc;
        Buffers &b = c->buf;
        b.cells_cap = (int)sc + c->cfg.n_dem_cells + 2;
        SPHDEM_CUDA_CHECK(cudaMalloc(&b.slot_z, capacity * sizeof(unsigned long long)));
        for (int **p : {&b.skey, &b.perm, &b.slot, &b.slot_tag, &b.key})
            SPHDEM_CUDA_CHECK(cudaMalloc(p, capacity * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&b.cnt, (size_t)b.cells_cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&b.start, ((size_t)b.cells_cap + 1) * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&b.fill, (size_t)b.cells_cap * sizeof(int)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&b.bsum, ((size_t)b.cells_cap / 4096 + 2) * sizeof(int)));
        setup_rebuild_buffers(c);
        if (cfg->flags & SPHDEM_F_CORRECTED_GRADIENT)
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->cg, (size_t)CG_ROWS * capacity * sizeof(double)));
        if (reinit_configured(*cfg)) SPHDEM_CUDA_CHECK(cudaMalloc(&c->hpred, capacity * sizeof(double)));
        SPHDEM_CUDA_CHECK(cudaMalloc(&c->delmark, capacity));
        SPHDEM_CUDA_CHECK(cudaMemset(c->delmark, 0, capacity));

        /* globals as the CdataLL constructor leaves them (dataLL.cpp:8-40) */
        DevGlobals hg;
        std::memset(&hg, 0, sizeof(hg));
        hg.dt = cfg->maxdt;
        hg.old_dt = cfg->maxdt;
        hg.maxdt = cfg->maxdt;
        hg.new_dt = cfg->maxdt;
        hg.dem_dt = cfg->maxdt;
        hg.sr = cfg->h;
        hg.hmax = cfg->h;
        for (int k = 0; k < 27; k++) hg.gw[k] = 1.1 * 2.0 * cfg->h;
        for (int d = 0; d < 3; d++) {
            hg.ghost_lo[d] = c->cfg.dmin[d] + hg.gw[0];
            double sp = c->cfg.dspace[d] - hg.gw[0];
            sp -= hg.gw[0];
            hg.ghost_sp[d] = sp;
            hg.ghost_rsp_f[d] = sp != 0 ? (float)(1.0 / sp) : 0.f;
        }
        SPHDEM_CUDA_CHECK(cudaMalloc(&c->dcfg, sizeof(DevCfg)));
        SPHDEM_CUDA_CHECK(cudaMemcpy(c->dcfg, &c->cfg, sizeof(DevCfg), cudaMemcpyHostToDevice));
        SPHDEM_CUDA_CHECK(cudaMalloc(&c->g, sizeof(DevGlobals)));
        SPHDEM_CUDA_CHECK(cudaMemcpy(c->g, &hg, sizeof(hg), cudaMemcpyHostToDevice));
        /* the uploads above ran on the legacy stream; the handle's stream is
         * non-blocking, so order them explicitly */
        SPHDEM_CUDA_CHECK(cudaDeviceSynchronize());
        run_h_derived(c);
        rebuild(c);
        if (cfg->precision == SPHDEM_PREC_MIXED) {
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_pos, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_vel, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_aux, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_tg, capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_om, capacity * sizeof(float)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_ncnt, capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_q0, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_q1, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_q2, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_dp, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_poslo, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_rc4, capacity * sizeof(int4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_shep32, capacity * sizeof(float)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_ds, capacity * sizeof(float4)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_nb, 3 * capacity * sizeof(float4)));
            c->mx_win_cap = win_cap;
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_win, 3 * (size_t)win_cap * sizeof(int4)));
            /* list entries that FP32 cannot decide (mostly FP64 ties: a staggered
             * lattice at rest density has 20 neighbours per particle at exactly
             * 2h) are recorded per particle for the FP64 fix-up pass */
            c->mx_band_per_particle = sphdem::mixed::band_records_per_particle();
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_bandq, capacity * c->mx_band_per_particle * sizeof(int2)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_bandn, capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMemset(c->mx_bandn, 0, capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMemset(c->mx_om, 0, capacity * sizeof(float)));
            SPHDEM_CUDA_CHECK(cudaMemset(c->mx_ncnt, 0, capacity * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaDeviceSynchronize());
            mixed::prepare(c);
            /* SPHDEM_FORCE_TILE=1: the force and continuity passes stage the
             * neighbour records in shared memory by bulk copies (measured
             * slower than reading them through L1 on the coupled workload,
             * so off by default) */
            const char *ft = std::getenv("SPHDEM_FORCE_TILE");
            c->force_tile = ft && ft[0] == '1';
            c->mx_dem_only = true;
            for (int64_t i = 0; i < init->n; i++) c->mx_dem_only = c->mx_dem_only && init->iam[i] == T_DEM;
            mixed::pack(c);
            const int m = mixed::nlist_max_count(c);
            if (m > 0) {
                /* headroom for compression; a run that outgrows it stops with
                 * SPHDEM_ERR_CAPACITY rather than dropping neighbours */
                int maxn = std::max(32, (int)(1.6 * m) + 16);
                maxn = (maxn + 31) / 32 * 32;
                c->mx_maxn = maxn;
                /* list tiles of 32 particles x 8 entries */
                SPHDEM_CUDA_CHECK(cudaMalloc(&c->mx_nbr, (size_t)maxn * ((capacity + 31) / 32 * 32) * sizeof(int)));
                /* the lists of the creation's rebuild, for exports before any step */
                mixed::nlist(c);
            }
        }
        int rc = check_device(c);
        if (rc != SPHDEM_OK) {
            g_create_err = c->err;
            fprintf(stderr, "sphdem_create: %s\n", c->err.c_str());
            free_ctx(c);
            return rc;
        }
    } catch (const std::string &e) {
        g_create_err = e;
        fprintf(stderr, "sphdem_create: %s\n", e.c_str());
        free_ctx(c);
        return SPHDEM_ERR_CUDA;
    }
    *out = c;
    return SPHDEM_OK;
}

int sphdem_destroy(sphdem_handle h) {
    if (!h) return SPHDEM_ERR_INVALID;
    collect_times(h);
    free_ctx(h);
    return SPHDEM_OK;
}

int sphdem_phase(sphdem_handle h, int phase) {
    if (!h) return SPHDEM_ERR_INVALID;
    if (phase < SPHDEM_HOOK_BEFORE_START || phase > SPHDEM_HOOK_AFTER_END)
        return fail(h, SPHDEM_ERR_INVALID, "unknown phase");
    try {
        run_phase(h, phase);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    const int rc = check_device(h);
    collect_times(h);
    return rc;
}

int sphdem_step(sphdem_handle h, int nsteps) {
    if (!h) return SPHDEM_ERR_INVALID;
    if (nsteps < 0) return fail(h, SPHDEM_ERR_INVALID, "negative step count");
    try {
        for (int k = 0; k < nsteps; k++) {
            if (h->timing) {
                run_full_step(h);
                continue;
            }
            /* a step that re-initialises the density rebuilds once more, so
             * it has its own graphs and may leave the other parity behind */
            const int key = (h->flipped ? 1 : 0) | (reinit_due(h->host_cfg, h->host_step + 1) ? 2 : 0);
            cudaGraphExec_t &ge = h->graph[key];
            if (!ge) {
                cudaGraph_t graph;
                h->in_capture = true;
                SPHDEM_CUDA_CHECK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
                run_full_step(h);   /* advances host_step and the parity */
                h->in_capture = false;
                SPHDEM_CUDA_CHECK(cudaStreamEndCapture(h->stream, &graph));
                h->graph_end_flip[key] = h->flipped;
                SPHDEM_CUDA_CHECK(cudaGraphInstantiate(&ge, graph, 0));
                cudaGraphDestroy(graph);
            } else {
                h->host_step++;
                if (h->flipped != h->graph_end_flip[key]) {
                    std::swap(h->A, h->B);
                    h->flipped = h->graph_end_flip[key];
                }
            }
            SPHDEM_CUDA_CHECK(cudaGraphLaunch(ge, h->stream));
        }
    } catch (const std::string &e) {
        h->in_capture = false;
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    const int rc = check_device(h);
    collect_times(h);
    return rc;
}

int sphdem_insert_particles(sphdem_handle h, const SphDemParticles *in, int64_t *out_idx) {
    if (!h || !in || in->n < 0) return SPHDEM_ERR_INVALID;
    if (in->n > 0 && (!in->iam || !in->r || !in->mass || !in->dens || !in->h))
        return fail(h, SPHDEM_ERR_INVALID, "iam, r, mass, dens and h are required");
    int rc;
    try {
        rc = insert_particles(h, in, out_idx);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return rc != SPHDEM_OK ? rc : check_device(h);
}

int sphdem_mark_for_deletion(sphdem_handle h, const int64_t *idx, int64_t k) {
    if (!h || k < 0 || (k > 0 && !idx)) return SPHDEM_ERR_INVALID;
    int rc;
    try {
        rc = mark_for_deletion(h, idx, k);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return rc != SPHDEM_OK ? rc : check_device(h);
}

int sphdem_rebuild(sphdem_handle h) {
    if (!h) return SPHDEM_ERR_INVALID;
    try {
        rebuild(h);
        if (h->mx_maxn > 0) {
            mixed::pack(h);
            mixed::nlist(h);
        }
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_time_steps(sphdem_handle h, int nsteps, double *ms) {
    if (!h || !ms) return SPHDEM_ERR_INVALID;
    int rc = sphdem_step(h, 1);  /* make sure the graph exists */
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, h->stream);
    rc = sphdem_step(h, nsteps);
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int sphdem_get_globals(sphdem_handle h, SphDemGlobals *out) {
    if (!h || !out) return SPHDEM_ERR_INVALID;
    DevGlobals hg;
    cudaStreamSynchronize(h->stream);
    if (cudaMemcpy(&hg, h->g, sizeof(hg), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(h, SPHDEM_ERR_CUDA, "cannot read globals");
    out->time = hg.time;
    out->dt = hg.dt;
    out->new_dt = hg.new_dt;
    out->maxdt = hg.maxdt;
    out->dem_dt = hg.dem_dt;
    out->sph_step = hg.step;
    out->n_deleted = hg.n_deleted;
    return SPHDEM_OK;
}

int sphdem_get_stats(sphdem_handle h, SphDemStats *out) {
    if (!h || !out) return SPHDEM_ERR_INVALID;
    cudaStreamSynchronize(h->stream);
    DevGlobals hg;
    cudaMemcpy(&hg, h->g, sizeof(hg), cudaMemcpyDeviceToHost);
    std::memset(out, 0, sizeof(*out));
    out->n_particles = h->n;
    std::vector<int> iam(h->n);
    cudaMemcpy(iam.data(), h->A.irow(FI_IAM), h->n * sizeof(int), cudaMemcpyDeviceToHost);
    for (int t : iam) out->n_alive += t != T_DEAD;
    if (h->mx_maxn > 0) {
        std::vector<int> cnt(h->n);
        cudaMemcpy(cnt.data(), h->mx_ncnt, h->n * sizeof(int), cudaMemcpyDeviceToHost);
        for (int64_t k = 0; k < h->n; k++)
            if (sphdem::is_sph_or_sphb(iam[k])) out->n_list_pairs += cnt[k];
    }
    out->list_depth = h->mx_maxn;
    out->n_sph_cells = hg.n_sph_cells;
    out->n_dem_cells = h->cfg.n_dem_cells;
    out->h_max = hg.hmax;
    out->search_radius = hg.sr;
    if (h->mx_bandn) {
        std::vector<int> nb(h->n);
        cudaMemcpy(nb.data(), h->mx_bandn, h->n * sizeof(int), cudaMemcpyDeviceToHost);
        for (int64_t k = 0; k < h->n; k++)
            if (sphdem::is_sph_or_sphb(iam[k])) out->n_band_candidates += nb[k];
        out->band_queue_capacity = (int64_t)h->cap * h->mx_band_per_particle;
    }
    return cudaGetLastError() == cudaSuccess ? SPHDEM_OK : SPHDEM_ERR_CUDA;
}

int sphdem_set_globals(sphdem_handle h, const SphDemGlobals *in) {
    if (!h || !in) return SPHDEM_ERR_INVALID;
    DevGlobals hg;
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(&hg, h->g, sizeof(hg), cudaMemcpyDeviceToHost);
    hg.time = in->time;
    hg.dt = in->dt;
    hg.maxdt = in->maxdt;
    hg.step = in->sph_step;
    if (cudaMemcpy(h->g, &hg, sizeof(hg), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(h, SPHDEM_ERR_CUDA, "cannot write globals");
    h->host_step = in->sph_step;
    cudaDeviceSynchronize();
    return SPHDEM_OK;
}

namespace {
struct FieldMap {
    uint32_t bit;
    int row;
    int ncomp;
    double *SphDemParticles::*ptr;
};
const FieldMap kFields[] = {
    {SPHDEM_FIELD_R, FD_R, 3, &SphDemParticles::r},
    {SPHDEM_FIELD_V, FD_V, 3, &SphDemParticles::v},
    {SPHDEM_FIELD_VHAT, FD_VHAT, 3, &SphDemParticles::vhat},
    {SPHDEM_FIELD_MASS, FD_MASS, 1, &SphDemParticles::mass},
    {SPHDEM_FIELD_DENS, FD_DENS, 1, &SphDemParticles::dens},
    {SPHDEM_FIELD_H, FD_H, 1, &SphDemParticles::h},
    {SPHDEM_FIELD_F, FD_F, 3, &SphDemParticles::f},
    {SPHDEM_FIELD_F, FD_FP, 3, &SphDemParticles::fp},
    {SPHDEM_FIELD_F, FD_FV, 3, &SphDemParticles::fv},
    {SPHDEM_FIELD_F, FD_FB, 3, &SphDemParticles::fb},
    {SPHDEM_FIELD_DDDT, FD_DDDT, 1, &SphDemParticles::dddt},
    {SPHDEM_FIELD_PRESS, FD_PRESS, 1, &SphDemParticles::press},
    {SPHDEM_FIELD_PRESS, FD_PDR2, 1, &SphDemParticles::pdr2},
    {SPHDEM_FIELD_COUPLING, FD_POR, 1, &SphDemParticles::porosity},
    {SPHDEM_FIELD_COUPLING, FD_DPORDT, 1, &SphDemParticles::dporositydt},
    {SPHDEM_FIELD_COUPLING, FD_SHEP, 1, &SphDemParticles::shep_sum},
    {SPHDEM_FIELD_COUPLING, FD_FDRAG, 3, &SphDemParticles::fdrag},
    {SPHDEM_FIELD_COUPLING, FD_FVEL, 3, &SphDemParticles::fvel},
    {SPHDEM_FIELD_COUPLING, FD_GPOR, 3, &SphDemParticles::grad_porosity},
    {SPHDEM_FIELD_OMEGA, FD_OMEGA, 1, &SphDemParticles::omega},
    {SPHDEM_FIELD_V0, FD_V0, 3, &SphDemParticles::v0},
    {SPHDEM_FIELD_V0, FD_VHAT0, 3, &SphDemParticles::vhat0},
    {SPHDEM_FIELD_NORMALS, FD_N1, 3, &SphDemParticles::norm1},
    {SPHDEM_FIELD_NORMALS, FD_N2, 3, &SphDemParticles::norm2},
    {SPHDEM_FIELD_NORMALS, FD_N3, 3, &SphDemParticles::norm3},
    {SPHDEM_FIELD_RADIUS, FD_RADIUS, 1, &SphDemParticles::radius},
    {SPHDEM_FIELD_ENERGY, FD_U, 1, &SphDemParticles::u},
    {SPHDEM_FIELD_ENERGY, FD_DUDT, 1, &SphDemParticles::dudt},
    {SPHDEM_FIELD_ENERGY, FD_EVISCF, 1, &SphDemParticles::e_visc},
    {SPHDEM_FIELD_ENERGY, FD_DEVISCF, 1, &SphDemParticles::de_visc_dt},
};
}  // namespace

int sphdem_get_fields(sphdem_handle h, uint32_t mask, SphDemParticles *out) {
    if (!h || !out) return SPHDEM_ERR_INVALID;
    if (out->n != h->n) return fail(h, SPHDEM_ERR_INVALID, "particle count mismatch");
    try {
        if (out->iam && (mask & SPHDEM_FIELD_IAM)) field_get_int(h, FI_IAM, out->iam);
        if (out->tag)
            for (int64_t k = 0; k < h->n; k++) out->tag[k] = (int32_t)(k + 1);
        for (const FieldMap &fm : kFields) {
            if (!(mask & fm.bit)) continue;
            double *dst = out->*fm.ptr;
            if (dst) field_get(h, fm.row, fm.ncomp, dst);
        }
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return SPHDEM_OK;
}

int sphdem_get_fields_async(sphdem_handle h, uint32_t mask, const SphDemParticles *out) {
    if (!h || !out) return SPHDEM_ERR_INVALID;
    if (out->n != h->n) return fail(h, SPHDEM_ERR_INVALID, "particle count mismatch");
    std::vector<FieldCopy> fc;
    for (const FieldMap &fm : kFields) {
        if (!(mask & fm.bit)) continue;
        double *dst = out->*fm.ptr;
        if (dst) fc.push_back(FieldCopy{fm.row, fm.ncomp, dst});
    }
    try {
        fields_get_async(h, fc.data(), (int)fc.size());
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return SPHDEM_OK;
}

int sphdem_fields_wait(sphdem_handle h) {
    if (!h) return SPHDEM_ERR_INVALID;
    try {
        fields_wait(h);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_set_fields(sphdem_handle h, uint32_t mask, const SphDemParticles *in) {
    if (!h || !in) return SPHDEM_ERR_INVALID;
    if (in->n != h->n) return fail(h, SPHDEM_ERR_INVALID, "particle count mismatch");
    try {
        for (const FieldMap &fm : kFields) {
            if (!(mask & fm.bit)) continue;
            const double *src = in->*fm.ptr;
            if (src) field_set(h, fm.row, fm.ncomp, src);
        }
        if (mask & SPHDEM_FIELD_H) run_h_derived(h);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_alloc_host(size_t bytes, void **ptr) {
    if (!ptr) return SPHDEM_ERR_INVALID;
    return cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) == cudaSuccess ? SPHDEM_OK : SPHDEM_ERR_CUDA;
}

int sphdem_free_host(void *ptr) {
    return cudaFreeHost(ptr) == cudaSuccess ? SPHDEM_OK : SPHDEM_ERR_CUDA;
}

int sphdem_pairs(sphdem_handle h, int kind, int64_t *offsets, int32_t *idx, int64_t idx_capacity, int64_t *n_pairs) {
    if (!h || !n_pairs || kind < 0 || kind > 3) return SPHDEM_ERR_INVALID;
    try {
        const int rc = export_pairs(h, kind, offsets, idx, idx_capacity, n_pairs);
        if (rc) return fail(h, rc, "pair buffer too small");
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return SPHDEM_OK;
}

int sphdem_cell_ids(sphdem_handle h, int32_t *cells) {
    if (!h || !cells) return SPHDEM_ERR_INVALID;
    try {
        const int rc = export_cells(h, cells);
        if (rc) return rc;
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_adjoint_forward(sphdem_handle h, int nsteps, int ckpt_every) {
    if (!h || nsteps <= 0 || ckpt_every <= 0) return SPHDEM_ERR_INVALID;
    try {
        int mode = 0;
        const std::string why = adjoint_supported(h, &mode);
        if (!why.empty()) return fail(h, SPHDEM_ERR_UNSUPPORTED, why);
        return adjoint_forward(h, nsteps, ckpt_every, mode);
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
}

int sphdem_adjoint_set_tape_memory(sphdem_handle h, int64_t bytes) {
    if (!h) return SPHDEM_ERR_INVALID;
    h->adj_tape_mem = bytes;
    return SPHDEM_OK;
}

int sphdem_adjoint_backward(sphdem_handle h, const double *dL_dr, const double *dL_dv, const double *dL_dvhat,
                            SphDemGrads *grads, double *dL_dr0, double *dL_dv0, double *dL_dvhat0) {
    if (!h || !grads) return SPHDEM_ERR_INVALID;
    std::memset(grads, 0, sizeof(*grads));
    try {
        double g5[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        uint32_t valid = 0;
        const int rc = adjoint_backward(h, dL_dr, dL_dv, dL_dvhat, g5, &valid, dL_dr0, dL_dv0, dL_dvhat0);
        if (rc == SPHDEM_ERR_CAPACITY) return fail(h, rc, "more pairs per step than the adjoint records");
        if (rc) return rc;
        grads->dem_k = g5[0];
        grads->dem_gamma = g5[1];
        /* the viscosity parameter of the handle's model: alpha_artificial
         * for artificial viscosity, the kinematic viscosity for Morris */
        grads->viscosity = h->cfg.visc == SPHDEM_VISC_ARTIFICIAL ? g5[2] : g5[3];
        grads->drag_scale = g5[4];
        grads->valid = valid;
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_output_vars(sphdem_handle h, SphDemOutputVars *out) {
    if (!h || !out) return SPHDEM_ERR_INVALID;
    try {
        const int rc = output_vars(h, out);
        if (rc) return rc;
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_cell_ids_noalloc(sphdem_handle h, int32_t *cells) {
    if (!h || !cells) return SPHDEM_ERR_INVALID;
    try {
        const int rc = export_cells_noalloc(h, cells);
        if (rc) return rc;
    } catch (const std::string &e) {
        return fail(h, SPHDEM_ERR_CUDA, e);
    }
    return check_device(h);
}

int sphdem_kernel_times_reset(sphdem_handle h, int enable) {
    if (!h) return SPHDEM_ERR_INVALID;
    collect_times(h);
    h->kt_names.clear();
    h->kt_ms.clear();
    h->kt_count.clear();
    h->timing = enable != 0;
    return SPHDEM_OK;
}

int sphdem_kernel_times(sphdem_handle h, char *names, size_t names_len, double *ms, int64_t *launches,
                        int max_kernels, int *n_kernels) {
    if (!h || !names || !ms || !launches || !n_kernels) return SPHDEM_ERR_INVALID;
    collect_times(h);
    std::string all;
    const int k = std::min<int>(max_kernels, (int)h->kt_names.size());
    for (int i = 0; i < k; i++) {
        if (i) all += "\n";
        all += h->kt_names[i];
        ms[i] = h->kt_ms[i];
        launches[i] = h->kt_count[i];
    }
    std::snprintf(names, names_len, "%s", all.c_str());
    *n_kernels = k;
    return SPHDEM_OK;
}

}  // extern "C"
