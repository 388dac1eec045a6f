/*
 * Host <-> device field transfer in tag order (the order particles were given
 * to sphdem_create), replacing the host-side particle container access of the
 * reference's hooks (particle.h Cparticle fields).  The device keeps particles
 * in bucket order; one kernel per field reorders through the tag row into a
 * staging buffer and one async copy moves it, so with pinned host memory a
 * field costs one pass over HBM and one copy.
 */
#include "internal.cuh"

namespace sphdem {
namespace {

__global__ void k_to_tag(const double *row, const int *tag, double *stage, int ncomp, int comp, int64_t n) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    stage[(int64_t)tag[k] * ncomp + comp] = row[k];
}

__global__ void k_from_tag(double *row, const int *tag, const double *stage, int ncomp, int comp, int64_t n) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    row[k] = stage[(int64_t)tag[k] * ncomp + comp];
}

__global__ void k_int_to_tag(const int *row, const int *tag, int *stage, int64_t n) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    stage[tag[k]] = row[k];
}

}  // namespace

void ensure_stage(sphdem_ctx *c) {
    if (!c->stage) SPHDEM_CUDA_CHECK(cudaMalloc(&c->stage, 3 * c->cap * sizeof(double)));
}

void field_get(sphdem_ctx *c, int row, int ncomp, double *host) {
    ensure_stage(c);
    const int64_t n = c->n;
    for (int d = 0; d < ncomp; d++)
        k_to_tag<<<grid_for(n, 256), 256, 0, c->stream>>>(c->A.row(row + d), c->A.irow(FI_TAG), c->stage, ncomp, d, n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(host, c->stage, ncomp * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
}

void field_set(sphdem_ctx *c, int row, int ncomp, const double *host) {
    ensure_stage(c);
    const int64_t n = c->n;
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(c->stage, host, ncomp * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    for (int d = 0; d < ncomp; d++)
        k_from_tag<<<grid_for(n, 256), 256, 0, c->stream>>>(c->A.row(row + d), c->A.irow(FI_TAG), c->stage, ncomp, d, n);
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
}

void fields_get_async(sphdem_ctx *c, const FieldCopy *fc, int nf) {
    const int64_t n = c->n;
    if (!c->copy_stream) {
        SPHDEM_CUDA_CHECK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            SPHDEM_CUDA_CHECK(cudaEventCreateWithFlags(&c->ev_gathered[k], cudaEventDisableTiming));
            SPHDEM_CUDA_CHECK(cudaEventCreateWithFlags(&c->ev_copied[k], cudaEventDisableTiming));
        }
    }
    size_t total = 0;
    for (int f = 0; f < nf; f++) total += (size_t)fc[f].ncomp * n;
    if (total == 0) return;
    const int b = c->acur;
    /* the previous copy out of this staging buffer must be done before it is
     * gathered into again */
    if (c->astage_used[b]) SPHDEM_CUDA_CHECK(cudaStreamWaitEvent(c->stream, c->ev_copied[b], 0));
    if (c->astage_cap[b] < total) {
        if (c->astage[b]) {
            SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->copy_stream));
            cudaFree(c->astage[b]);
            c->astage[b] = nullptr;
        }
        SPHDEM_CUDA_CHECK(cudaMalloc(&c->astage[b], total * sizeof(double)));
        c->astage_cap[b] = total;
    }
    double *st = c->astage[b];
    size_t off = 0;
    for (int f = 0; f < nf; f++) {
        for (int d = 0; d < fc[f].ncomp; d++)
            k_to_tag<<<grid_for(n, 256), 256, 0, c->stream>>>(c->A.row(fc[f].row + d), c->A.irow(FI_TAG), st + off,
                                                             fc[f].ncomp, d, n);
        off += (size_t)fc[f].ncomp * n;
    }
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    SPHDEM_CUDA_CHECK(cudaEventRecord(c->ev_gathered[b], c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamWaitEvent(c->copy_stream, c->ev_gathered[b], 0));
    off = 0;
    for (int f = 0; f < nf; f++) {
        const size_t bytes = (size_t)fc[f].ncomp * n * sizeof(double);
        SPHDEM_CUDA_CHECK(cudaMemcpyAsync(fc[f].host, st + off, bytes, cudaMemcpyDeviceToHost, c->copy_stream));
        off += (size_t)fc[f].ncomp * n;
    }
    SPHDEM_CUDA_CHECK(cudaEventRecord(c->ev_copied[b], c->copy_stream));
    c->astage_used[b] = true;
    c->acur = b ^ 1;
}

void fields_wait(sphdem_ctx *c) {
    if (c->copy_stream) SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->copy_stream));
}

void fields_async_free(sphdem_ctx *c) {
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (int k = 0; k < 2; k++) {
        cudaFree(c->astage[k]);
        if (c->ev_gathered[k]) cudaEventDestroy(c->ev_gathered[k]);
        if (c->ev_copied[k]) cudaEventDestroy(c->ev_copied[k]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
}

void field_get_int(sphdem_ctx *c, int row, int *host) {
    ensure_stage(c);
    const int64_t n = c->n;
    int *st = reinterpret_cast<int *>(c->stage);
    k_int_to_tag<<<grid_for(n, 256), 256, 0, c->stream>>>(c->A.irow(row), c->A.irow(FI_TAG), st, n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(host, st, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
}

}  // namespace sphdem
