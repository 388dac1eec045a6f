/*
 * Particle insertion and deletion between phases: CdataLL::insertNewParticle
 * (dataLL.cpp:238-261) and CdataLL::markForDeletion (dataLL.cpp:263-266),
 * whose marked particles leave at the next reset (updateDomain,
 * dataLL.cpp:377-380).
 *
 * Indices are tag-order indices (the order of sphdem_create, then of
 * insertion).  A deleted particle keeps its index as a dead slot (type
 * T_DEAD, sorted into the dead bucket by every rebuild); an insertion takes
 * the lowest dead slot first and appends past the last index only when none
 * is left, so a run with inflow and outflow stays within the capacity given
 * at creation.  The new rows are written where the slot's particle sits in
 * the current (bucket-sorted) state; the next rebuild sorts them in, and
 * every neighbour pass of a phase follows that phase's rebuild.
 */
#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 256;

/* pos[tag] = state position of that tag */
__global__ void k_pos_of_tag(const int *tag, int *pos, int64_t n) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n) pos[tag[p]] = (int)p;
}

__global__ void k_mark(const int *pos, const int64_t *idx, int64_t k, unsigned char *mark) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j < k) mark[pos[idx[j]]] = 1;
}

/* One new particle per thread.  blk holds INS_ND doubles per particle
 * (r, v, vhat, norm1..3: 3 each; mass, dens, h, radius), ints holds iam and
 * concave.  Every other row starts as sphdem_create leaves it: zero, with
 * porosity 1 (Cparticle(), particle.h:82). */
enum : int { IB_R = 0, IB_V = 3, IB_VH = 6, IB_N1 = 9, IB_N2 = 12, IB_N3 = 15, IB_MASS = 18, IB_DENS, IB_H, IB_RAD,
             INS_ND };

__global__ void k_insert(DevCfg c, DevState s, const int *pos, const int64_t *slot, const double *blk,
                         const int *ints, int64_t k, int64_t n_old, unsigned char *mark) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= k) return;
    const int64_t t = slot[j];
    const int64_t p = t < n_old ? pos[t] : t;
    for (int f = 0; f < NFD; f++) s.row(f)[p] = 0.0;
    for (int f = 0; f < NFI; f++) s.irow(f)[p] = 0;
    const double *b = blk + j * INS_ND;
    for (int d = 0; d < 3; d++) {
        s.row(FD_R + d)[p] = b[IB_R + d];
        s.row(FD_V + d)[p] = b[IB_V + d];
        s.row(FD_VHAT + d)[p] = b[IB_VH + d];
        s.row(FD_N1 + d)[p] = b[IB_N1 + d];
        s.row(FD_N2 + d)[p] = b[IB_N2 + d];
        s.row(FD_N3 + d)[p] = b[IB_N3 + d];
    }
    s.row(FD_MASS)[p] = b[IB_MASS];
    s.row(FD_DENS)[p] = b[IB_DENS];
    s.row(FD_H)[p] = b[IB_H];
    s.row(FD_RADIUS)[p] = b[IB_RAD];
    s.row(FD_POR)[p] = 1.0;
    h_derived(c, s, p);
    s.irow(FI_IAM)[p] = ints[2 * j];
    s.irow(FI_CONCAVE)[p] = ints[2 * j + 1];
    s.irow(FI_TAG)[p] = (int)t;
    mark[p] = 0;
}

/* graphs and adjoint tapes hold the particle count: drop them */
void population_changed(sphdem_ctx *c) {
    for (int k = 0; k < 4; k++) {
        if (c->graph[k]) cudaGraphExecDestroy(c->graph[k]);
        c->graph[k] = nullptr;
    }
    if (c->adj) adjoint_free(c);
    c->population_gen++;
}

}  // namespace

int insert_particles(sphdem_ctx *c, const SphDemParticles *in, int64_t *out_idx) {
    const int64_t k = in->n;
    if (k == 0) return SPHDEM_OK;
    const int64_t n_old = c->n;
    /* free slots: dead particles, lowest index first */
    std::vector<int> iam(n_old);
    field_get_int(c, FI_IAM, iam.data());
    std::vector<int64_t> slot(k);
    int64_t next = n_old, cursor = 0;
    for (int64_t j = 0; j < k; j++) {
        while (cursor < n_old && iam[cursor] != T_DEAD) cursor++;
        slot[j] = cursor < n_old ? cursor++ : next++;
    }
    if (next > c->cap) {
        c->err = "insertion beyond the capacity given at creation (" + std::to_string(next) + " > " +
                 std::to_string(c->cap) + ")";
        return SPHDEM_ERR_CAPACITY;
    }
    if (next > ((int64_t)1 << 26)) {
        c->err = "insertion beyond 2^26 particles";
        return SPHDEM_ERR_CAPACITY;
    }
    std::vector<double> blk((size_t)k * INS_ND);
    std::vector<int> ints((size_t)k * 2);
    for (int64_t j = 0; j < k; j++) {
        double *b = blk.data() + j * INS_ND;
        for (int d = 0; d < 3; d++) {
            b[IB_R + d] = in->r[3 * j + d];
            b[IB_V + d] = in->v ? in->v[3 * j + d] : 0.0;
            b[IB_VH + d] = in->vhat ? in->vhat[3 * j + d] : b[IB_V + d];
            b[IB_N1 + d] = in->norm1 ? in->norm1[3 * j + d] : 0.0;
            b[IB_N2 + d] = in->norm2 ? in->norm2[3 * j + d] : 0.0;
            b[IB_N3 + d] = in->norm3 ? in->norm3[3 * j + d] : 0.0;
        }
        b[IB_MASS] = in->mass[j];
        b[IB_DENS] = in->dens[j];
        b[IB_H] = in->h[j];
        b[IB_RAD] = in->radius ? in->radius[j] : 0.0;
        ints[2 * j] = in->iam[j];
        ints[2 * j + 1] = in->concave ? in->concave[j] != 0 : 1;
    }
    double *d_blk = nullptr;
    int *d_ints = nullptr;
    int64_t *d_slot = nullptr;
    SPHDEM_CUDA_CHECK(cudaMallocAsync(&d_blk, blk.size() * sizeof(double), c->stream));
    SPHDEM_CUDA_CHECK(cudaMallocAsync(&d_ints, ints.size() * sizeof(int), c->stream));
    SPHDEM_CUDA_CHECK(cudaMallocAsync(&d_slot, slot.size() * sizeof(int64_t), c->stream));
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(d_blk, blk.data(), blk.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(d_ints, ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    SPHDEM_CUDA_CHECK(
        cudaMemcpyAsync(d_slot, slot.data(), slot.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    int *pos = c->buf.slot;   /* rebuild scratch, free between rebuilds */
    if (n_old > 0) k_pos_of_tag<<<grid_for(n_old, BLK), BLK, 0, c->stream>>>(c->A.irow(FI_TAG), pos, n_old);
    k_insert<<<grid_for(k, BLK), BLK, 0, c->stream>>>(c->cfg, c->A, pos, d_slot, d_blk, d_ints, k, n_old, c->delmark);
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    SPHDEM_CUDA_CHECK(cudaFreeAsync(d_blk, c->stream));
    SPHDEM_CUDA_CHECK(cudaFreeAsync(d_ints, c->stream));
    SPHDEM_CUDA_CHECK(cudaFreeAsync(d_slot, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    c->n = next;
    population_changed(c);
    if (out_idx) std::copy(slot.begin(), slot.end(), out_idx);
    return SPHDEM_OK;
}

int mark_for_deletion(sphdem_ctx *c, const int64_t *idx, int64_t k) {
    if (k == 0) return SPHDEM_OK;
    std::vector<int> iam(c->n);
    field_get_int(c, FI_IAM, iam.data());
    for (int64_t j = 0; j < k; j++) {
        if (idx[j] < 0 || idx[j] >= c->n) {
            c->err = "deletion index " + std::to_string(idx[j]) + " out of range";
            return SPHDEM_ERR_INVALID;
        }
        if (iam[idx[j]] == T_DEAD) {
            c->err = "deletion of particle " + std::to_string(idx[j]) + ", which is already deleted";
            return SPHDEM_ERR_INVALID;
        }
    }
    int64_t *d_idx = nullptr;
    SPHDEM_CUDA_CHECK(cudaMallocAsync(&d_idx, k * sizeof(int64_t), c->stream));
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(d_idx, idx, k * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    int *pos = c->buf.slot;
    k_pos_of_tag<<<grid_for(c->n, BLK), BLK, 0, c->stream>>>(c->A.irow(FI_TAG), pos, c->n);
    k_mark<<<grid_for(k, BLK), BLK, 0, c->stream>>>(pos, d_idx, k, c->delmark);
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    SPHDEM_CUDA_CHECK(cudaFreeAsync(d_idx, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    return SPHDEM_OK;
}

}  // namespace sphdem
