/*
 * Output-step diagnostics on the device: CsphIncompress::calcOutputVars
 * (sphIncompress.h:274-319) with calcOutput (233-262), calcVarDens (264) and
 * calcAveDensFromMass (266-272, which sums calcDensity, sph.h:1149-1191, over
 * each particle's neighbours).
 *
 * One grid-stride pass accumulates per-block FP64 partial sums and maxima of
 * every quantity; the host adds the partials in block order (deterministic).
 * A second pass sums (rho - <rho>)^2 for varDens.  The density summation
 * scans the buckets of the last rebuild with the exact neighbour predicate
 * (particle.h:236-238), as the reference's cached lists hold the neighbours
 * of that reset.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int OB = 256;
constexpr int OG = 608;  /* blocks: 4 per SM on 152 SMs */

enum : int {
    OS_LINX = 0, OS_LINY, OS_LINZ, OS_ANG, OS_KE, OS_VISCF, OS_DVISCF, OS_NSPH, OS_DENS, OS_ELAST, OS_DELAST,
    OS_EXACT, OS_DFM, OS_N, OS_NSUM
};
enum : int { OM_V = 0, OM_F, OS_NMAX };

__device__ __forceinline__ double kernel_k(double q, double wcon) {
    if (q > 2.0) return 0.0;
    const double t = 2.0 - q, t2 = t * t;
    return wcon * (t2 * t2) * (1.0 + 2.0 * q);
}

/* calcDensity (non-MLS): m_a W(0, h_a) + sum over sph / sphBoundary
 * neighbours of m_b W(r / h_a, h_a) */
__device__ double density_sum(const DevCfg &c, const DevState &s, const int *start, const int *skey,
                              const DevGlobals *g, int64_t a) {
    const GridInfo gi = load_grid(g);
    const CellCoord cc = decode_cell(skey[a], gi.sdims, c.nd);
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ha = s.row(FD_H)[a], iha = 1.0 / ha;
    double ihn = 1.0;
    for (int d = 0; d < c.nd; d++) ihn *= iha;
    double rho = s.row(FD_MASS)[a] * ihn * kernel_k(0.0, c.wcon);
    scan_cells(cc, gi.sdims, c.periodic, c.nd, start, 0, [&](int b, const int *sh) {
        const bool shifted = (sh[0] | sh[1] | sh[2]) != 0;
        if (b == a && !shifted) return;
        if (!is_sph_or_sphb(s.irow(FI_IAM)[b])) return;
        double dx[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++)
            dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
        const double r2 = exact_len2(dx, c.nd);
        const double hb = s.row(FD_H)[b];
        const double t = 2.0 * (ha > hb ? ha : hb);
        if (r2 > dmul(t, t)) return;
        if (shifted && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return;
        rho += s.row(FD_MASS)[b] * ihn * kernel_k(sqrt(r2) * iha, c.wcon);
    });
    return rho;
}

__device__ __forceinline__ void block_sum(double *sh, double v, double *out) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sh[k];
        *out = t;
    }
}

__device__ __forceinline__ void block_max(double *sh, double v, double *out) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t = fmax(t, sh[k]);
        *out = t;
    }
}

__global__ void k_output_vars(DevCfg c, DevState s, const int *start, const int *skey, const DevGlobals *g,
                              int64_t n, double *part_sum, double *part_max) {
    __shared__ double shm[32];
    double acc[OS_NSUM], mx[OS_NMAX];
    for (int k = 0; k < OS_NSUM; k++) acc[k] = 0.0;
    for (int k = 0; k < OS_NMAX; k++) mx[k] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int t = s.irow(FI_IAM)[i];
        if (t == T_DEAD) continue;
        acc[OS_N] += 1.0;
        if (!is_sph_or_sphb(t)) continue;
        const double m = s.row(FD_MASS)[i], dens = s.row(FD_DENS)[i];
        double v2 = 0.0, f2 = 0.0, vh2 = 0.0;
        for (int d = 0; d < c.nd; d++) {
            const double v = s.row(FD_V + d)[i], f = s.row(FD_F + d)[i], vh = s.row(FD_VHAT + d)[i];
            v2 += v * v;
            f2 += f * f;
            vh2 += vh * vh;
        }
        if (t == T_SPH) {
            for (int d = 0; d < c.nd; d++) acc[OS_LINX + d] += s.row(FD_V + d)[i] * m;
            /* the reference's 2D angular momentum (x v_y - y v_x) m in every dimension */
            acc[OS_ANG] += (s.row(FD_R)[i] * s.row(FD_V + 1)[i] - s.row(FD_R + 1)[i] * s.row(FD_V)[i]) * m;
            acc[OS_KE] += 0.5 * m * vh2;
            acc[OS_VISCF] += m * s.row(FD_EVISCF)[i];
            acc[OS_DVISCF] += m * s.row(FD_DEVISCF)[i];
            acc[OS_NSPH] += 1.0;
        }
        mx[OM_V] = fmax(mx[OM_V], sqrt(v2));
        mx[OM_F] = fmax(mx[OM_F], sqrt(f2));
        acc[OS_DENS] += dens;
        acc[OS_ELAST] += m * s.row(FD_U)[i];
        acc[OS_DELAST] += m * s.row(FD_DUDT)[i];
        const double x = dens / c.refd, x2 = x * x;
        acc[OS_EXACT] += m * (c.prb * ((x2 * x2 * x2 - 1.0) / 6.0 + 1.0 / x - 1.0)) / c.refd;
        const double dr = density_sum(c, s, start, skey, g, i) - dens;
        acc[OS_DFM] += dr * dr;
    }
    for (int k = 0; k < OS_NSUM; k++) block_sum(shm, acc[k], part_sum + (int64_t)blockIdx.x * OS_NSUM + k);
    for (int k = 0; k < OS_NMAX; k++) block_max(shm, mx[k], part_max + (int64_t)blockIdx.x * OS_NMAX + k);
}

__global__ void k_var_dens(DevState s, int64_t n, double ave, double *part) {
    __shared__ double shm[32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!is_sph_or_sphb(s.irow(FI_IAM)[i])) continue;
        const double d = s.row(FD_DENS)[i] - ave;
        acc += d * d;
    }
    block_sum(shm, acc, part + blockIdx.x);
}

}  // namespace

int output_vars(sphdem_ctx *c, SphDemOutputVars *o) {
    double *part = nullptr;
    const size_t nb = (size_t)OG * (OS_NSUM + OS_NMAX + 1);
    SPHDEM_CUDA_CHECK(cudaMallocAsync(&part, nb * sizeof(double), c->stream));
    double *ps = part, *pm = part + (size_t)OG * OS_NSUM, *pv = pm + (size_t)OG * OS_NMAX;
    k_output_vars<<<OG, OB, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->buf.skey, c->g, c->n, ps, pm);
    std::vector<double> h((size_t)OG * (OS_NSUM + OS_NMAX));
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    double sum[OS_NSUM] = {0}, mx[OS_NMAX] = {0};
    for (int b = 0; b < OG; b++) {
        for (int k = 0; k < OS_NSUM; k++) sum[k] += h[(size_t)b * OS_NSUM + k];
        for (int k = 0; k < OS_NMAX; k++) mx[k] = std::max(mx[k], h[(size_t)OG * OS_NSUM + (size_t)b * OS_NMAX + k]);
    }
    const double n = sum[OS_N];
    const double ave = n > 0 ? sum[OS_DENS] / n : 0.0;
    k_var_dens<<<OG, OB, 0, c->stream>>>(c->A, c->n, ave, pv);
    std::vector<double> hv(OG);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(hv.data(), pv, OG * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaFreeAsync(part, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    double var = 0.0;
    for (int b = 0; b < OG; b++) var += hv[b];
    *o = SphDemOutputVars{};
    for (int d = 0; d < 3; d++) o->lin_mom[d] = sum[OS_LINX + d];
    o->ang_mom = sum[OS_ANG];
    o->e_ke = sum[OS_KE];
    o->e_visc_f = sum[OS_VISCF];
    o->ed_visc_f_dt = sum[OS_DVISCF];
    o->e_elast = sum[OS_ELAST];
    o->ed_elast_dt = sum[OS_DELAST];
    o->e_elast_exact = sum[OS_EXACT];
    o->e_ff = o->ed_ff_dt = o->e_visc_b = o->e_b_force = 0.0;   /* ff, eViscB, eBForce are 0 on this path */
    o->max_v = mx[OM_V];
    o->max_f = mx[OM_F];
    o->max_ff = 0.0;
    o->rms_ff = 0.0;
    o->n = (int64_t)n;
    o->n_sph = (int64_t)sum[OS_NSPH];
    o->ave_dens = ave;
    o->ave_dens_from_mass = n > 0 ? std::sqrt(sum[OS_DFM] / n) : 0.0;
    o->var_dens = n > 0 ? var / n : 0.0;
    o->e_total = o->e_ke + o->e_elast + o->e_visc_f + o->e_visc_b + o->e_b_force + o->e_ff;
    return SPHDEM_OK;
}

}  // namespace sphdem
