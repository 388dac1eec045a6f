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

void field_get_int(sphdem_ctx *c, int row, int *host) {
    ensure_stage(c);
    const int64_t n = c->n;
    int *st = reinterpret_cast<int *>(c->stage);
    k_int_to_tag<<<grid_for(n, 256), 256, 0, c->stream>>>(c->A.irow(row), c->A.irow(FI_TAG), st, n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(host, st, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
}

}  // namespace sphdem
