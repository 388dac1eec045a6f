/*
 * Batched ensembles: many independent simulations (handles of any size)
 * stepped together by one CUDA graph per step.
 *
 * The graph is captured by forking the batch stream into every member's
 * stream, recording each member's full step there, and joining back: the
 * members' kernel chains become independent branches of one graph, so one
 * cudaGraphLaunch per step keeps the GPU filled with the small grids of many
 * small simulations at once.  Members keep their own state, globals, time
 * step and error flags; nothing is shared between them.
 *
 * The autotuner (sphdem_batch_tune) picks, per member, the block size of the
 * list-consumer passes, the grid of the slice passes and whether the force
 * and continuity passes stage their neighbour tiles in shared memory, by
 * timing a few graph-replayed steps of that member alone for every
 * candidate; the choice is remembered per dimension, precision, feature
 * flags and particle-count octave, and members of a class tuned before
 * take it without timing.
 *
 * The reference runs one simulation per process; this file has no
 * counterpart there.
 */
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"

struct sphdem_batch_ctx {
    std::vector<sphdem_ctx *> members;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<char> graph_parity;   /* members' buffer parity the graph was captured at */
    std::vector<long long> graph_gen; /* members' population generation at capture */
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev_join;
    std::string err;
};

namespace {

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::string(what) + ": " + cudaGetErrorString(e);
}

/* the batch stream waits for every member's pending work */
void join_members_into_batch(sphdem_batch_ctx *b) {
    for (size_t i = 0; i < b->members.size(); i++) {
        check_cuda(cudaEventRecord(b->ev_join[i], b->members[i]->stream), "record member event");
        check_cuda(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0), "batch waits for member");
    }
}

/* every member stream waits for the batch stream */
void release_members(sphdem_batch_ctx *b) {
    check_cuda(cudaEventRecord(b->ev_fork, b->stream), "record batch event");
    for (sphdem_ctx *m : b->members) check_cuda(cudaStreamWaitEvent(m->stream, b->ev_fork, 0), "member waits");
}

void drop_graph(sphdem_batch_ctx *b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

void capture(sphdem_batch_ctx *b) {
    drop_graph(b);
    cudaGraph_t graph = nullptr;
    check_cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
        check_cuda(cudaEventRecord(b->ev_fork, b->stream), "fork");
        for (size_t i = 0; i < b->members.size(); i++) {
            sphdem_ctx *m = b->members[i];
            check_cuda(cudaStreamWaitEvent(m->stream, b->ev_fork, 0), "fork wait");
            m->in_capture = true;
            const bool p0 = m->flipped;
            sphdem::step_sequence(m);
            m->in_capture = false;
            if (m->flipped != p0) throw std::string("a step must rebuild an even number of times");
            check_cuda(cudaEventRecord(b->ev_join[i], m->stream), "join record");
            check_cuda(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0), "join wait");
        }
    } catch (...) {
        for (sphdem_ctx *m : b->members) m->in_capture = false;
        cudaStreamEndCapture(b->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    check_cuda(cudaStreamEndCapture(b->stream, &graph), "end capture");
    const cudaError_t e = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    check_cuda(e, "instantiate");
    b->graph_parity.resize(b->members.size());
    b->graph_gen.resize(b->members.size());
    for (size_t i = 0; i < b->members.size(); i++) {
        b->graph_parity[i] = b->members[i]->flipped;
        b->graph_gen[i] = b->members[i]->population_gen;
    }
}

bool parity_changed(const sphdem_batch_ctx *b) {
    if (!b->graph) return true;
    for (size_t i = 0; i < b->members.size(); i++)
        if ((char)b->members[i]->flipped != b->graph_parity[i] ||
            b->members[i]->population_gen != b->graph_gen[i])
            return true;
    return false;
}

int batch_fail(sphdem_batch_ctx *b, int code, const std::string &msg) {
    b->err = msg;
    return code;
}

/* device error flags of every member (synchronises) */
int check_members(sphdem_batch_ctx *b) {
    check_cuda(cudaStreamSynchronize(b->stream), "batch stream");
    for (size_t i = 0; i < b->members.size(); i++) {
        const int rc = sphdem::device_status(b->members[i]);
        if (rc != SPHDEM_OK) return batch_fail(b, rc, "member " + std::to_string(i) + ": " + b->members[i]->err);
    }
    return SPHDEM_OK;
}

}  // namespace

extern "C" {

/* text of the calling thread's last failed sphdem_batch_create */
static thread_local std::string g_batch_create_err;

int sphdem_batch_create(const sphdem_handle *members, int n, sphdem_batch *out) {
    auto bad = [](int code, const std::string &msg) {
        g_batch_create_err = msg;
        return code;
    };
    if (!out) return bad(SPHDEM_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (!members || n <= 0) return bad(SPHDEM_ERR_INVALID, "no members");
    for (int i = 0; i < n; i++)
        if (!members[i]) return bad(SPHDEM_ERR_INVALID, "member " + std::to_string(i) + " is a null handle");
    for (int i = 0; i < n; i++)
        for (int j = 0; j < i; j++)
            if (members[i] == members[j])
                return bad(SPHDEM_ERR_INVALID,
                           "members " + std::to_string(j) + " and " + std::to_string(i) + " are the same handle");
    /* a density re-initialisation step rebuilds once more than the others,
     * which one shared graph per step cannot follow */
    for (int i = 0; i < n; i++)
        if (sphdem::reinit_configured(members[i]->host_cfg))
            return bad(SPHDEM_ERR_UNSUPPORTED,
                       "member " + std::to_string(i) + " re-initialises its density (reinit_dens_every / reinit_dens_at)");
    sphdem_batch_ctx *b = new sphdem_batch_ctx;
    b->members.assign(members, members + n);
    b->ev_join.assign(n, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->ev_join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        sphdem_batch_destroy(b);
        return bad(SPHDEM_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
    }
    *out = b;
    return SPHDEM_OK;
}

int sphdem_batch_destroy(sphdem_batch b) {
    if (!b) return SPHDEM_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (cudaEvent_t e : b->ev_join)
        if (e) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SPHDEM_OK;
}

int sphdem_batch_step(sphdem_batch b, int nsteps) {
    if (!b || nsteps < 0) return SPHDEM_ERR_INVALID;
    try {
        join_members_into_batch(b);
        for (int k = 0; k < nsteps; k++) {
            if (parity_changed(b)) capture(b);
            check_cuda(cudaGraphLaunch(b->graph, b->stream), "graph launch");
        }
        release_members(b);
    } catch (const std::string &e) {
        return batch_fail(b, SPHDEM_ERR_CUDA, e);
    }
    return check_members(b);
}

int sphdem_batch_time_steps(sphdem_batch b, int nsteps, double *ms) {
    if (!b || !ms || nsteps < 0) return SPHDEM_ERR_INVALID;
    int rc = sphdem_batch_step(b, 1); /* the graph exists and every member is in step */
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    try {
        check_cuda(cudaEventCreate(&e0), "event");
        check_cuda(cudaEventCreate(&e1), "event");
        join_members_into_batch(b);
        check_cuda(cudaEventRecord(e0, b->stream), "record");
        for (int k = 0; k < nsteps; k++) check_cuda(cudaGraphLaunch(b->graph, b->stream), "graph launch");
        check_cuda(cudaEventRecord(e1, b->stream), "record");
        release_members(b);
        check_cuda(cudaEventSynchronize(e1), "sync");
        float t = 0.f;
        check_cuda(cudaEventElapsedTime(&t, e0, e1), "elapsed");
        *ms = t;
    } catch (const std::string &e) {
        rc = batch_fail(b, SPHDEM_ERR_CUDA, e);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc ? rc : check_members(b);
}

/* Tuned launch shapes, remembered per (dimension, precision, feature flags,
 * particle-count octave) for the rest of the process: a member whose class
 * was tuned before takes the same shape without timing. */
struct TuneKey {
    int nd, precision;
    unsigned flags;
    int octave;
    bool operator<(const TuneKey &o) const {
        if (nd != o.nd) return nd < o.nd;
        if (precision != o.precision) return precision < o.precision;
        if (flags != o.flags) return flags < o.flags;
        return octave < o.octave;
    }
};
struct TuneChoice {
    int blk, div, tile;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune_cache;

void drop_member_graphs(sphdem_ctx *m) {
    for (cudaGraphExec_t &g : m->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

int sphdem_batch_tune(sphdem_batch b, int steps_per_trial, int *chosen) {
    if (!b || steps_per_trial <= 0) return SPHDEM_ERR_INVALID;
    static const int blk_opts[] = {64, 128};
    static const int div_opts[] = {1, 4};
    try {
        drop_graph(b);
        for (size_t i = 0; i < b->members.size(); i++) {
            sphdem_ctx *m = b->members[i];
            int octave = 0;
            while ((int64_t(1) << (octave + 1)) <= m->n) octave++;
            const TuneKey key{m->cfg.nd, m->cfg.precision, m->host_cfg.flags, octave};
            TuneChoice best_c{m->blk_pair, m->grid_div, m->force_tile ? 1 : 0};
            bool cached = false;
            {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                auto it = g_tune_cache.find(key);
                if (it != g_tune_cache.end()) {
                    best_c = it->second;
                    cached = true;
                }
            }
            if (!cached) {
                /* staged neighbour tiles apply to the list passes of mixed
                 * handles in 2D and 3D */
                const int tiles = (m->cfg.precision == SPHDEM_PREC_MIXED && m->cfg.nd > 1 && m->mx_maxn > 0) ? 2 : 1;
                double best = 1e300;
                for (int blk : blk_opts)
                    for (int dv : div_opts)
                        for (int tl = 0; tl < tiles; tl++) {
                            m->blk_pair = blk;
                            m->grid_div = dv;
                            m->force_tile = tl != 0;
                            drop_member_graphs(m);
                            double ms = 0.0;
                            const int rc = sphdem_time_steps(m, steps_per_trial, &ms);
                            if (rc) return batch_fail(b, rc, "tuning member " + std::to_string(i) + ": " + m->err);
                            if (ms < best) {
                                best = ms;
                                best_c = TuneChoice{blk, dv, tl};
                            }
                        }
                std::lock_guard<std::mutex> lock(g_tune_mu);
                g_tune_cache[key] = best_c;
            }
            m->blk_pair = best_c.blk;
            m->grid_div = best_c.div;
            m->force_tile = best_c.tile != 0;
            drop_member_graphs(m);
            if (chosen) {
                chosen[3 * i] = best_c.blk;
                chosen[3 * i + 1] = best_c.div;
                chosen[3 * i + 2] = best_c.tile;
            }
        }
    } catch (const std::string &e) {
        return batch_fail(b, SPHDEM_ERR_CUDA, e);
    }
    return SPHDEM_OK;
}

int sphdem_batch_last_error(sphdem_batch b, char *buf, size_t len) {
    if (!buf || !len) return SPHDEM_ERR_INVALID;
    const std::string e = b ? b->err : (g_batch_create_err.empty() ? std::string("no batch") : g_batch_create_err);
    std::snprintf(buf, len, "%s", e.c_str());
    return SPHDEM_OK;
}

}  // extern "C"
