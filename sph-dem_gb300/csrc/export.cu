/*
 * Parity exports: the neighbour relations (calcNeighbours, dataLL.cpp:1026-1075;
 * calcNeighboursCoupling, dataLL.cpp:1104-1192) and the reference bucket index
 * of every particle (getCellI / dem_getCellI, dataLL.h:303-311), in tag order.
 * They read the bucket lists of the last rebuild, like the reference's own
 * lists after a reset.
 */
#include <algorithm>

#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 128;

__device__ __forceinline__ CellCoord cell_sph(const DevCfg &c, const DevGlobals *g, const double *r) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    for (int d = 0; d < c.nd; d++) {
        int k = c.periodic[d] ? (int)floor((r[d] - c.dmin[d]) * g->rscell[d])
                              : trunc_index(r[d], c.dmin[d], g->sr2, g->rsr2_f, 3.0);
        k = k < 0 ? 0 : (k >= g->sdims[d] ? g->sdims[d] - 1 : k);
        cc.c[d] = k;
    }
    return cc;
}

__device__ __forceinline__ CellCoord cell_dem(const DevCfg &c, const double *r) {
    CellCoord cc;
    cc.c[0] = cc.c[1] = cc.c[2] = 0;
    for (int d = 0; d < c.nd; d++) {
        int k = (int)floor((r[d] - c.dorig[d]) * c.rdcell[d]);
        if (k < 0) k = c.periodic[d] ? c.ddims[d] - 1 : 0;
        if (k >= c.ddims[d]) k = c.periodic[d] ? 0 : c.ddims[d] - 1;
        cc.c[d] = k;
    }
    return cc;
}

/* mode 0: count, 1: write (tag-order rows at offs[tag]) */
__global__ void k_pairs(DevCfg c, DevState s, const int *start, const DevGlobals *g, int64_t n, int kind,
                        int mode, int *cnt, const long long *offs, int *idx, int skip_listed) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int ta = s.irow(FI_IAM)[a];
    if (ta == T_DEAD) return;
    if (skip_listed && is_sph_or_sphb(ta)) return;  /* these rows come from the neighbour lists */
    const bool dem = c.liq_dem() && ta == T_DEM;
    const int tag = s.irow(FI_TAG)[a];
    double ra[3] = {0, 0, 0};
    for (int d = 0; d < c.nd; d++) ra[d] = s.row(FD_R + d)[a];
    const double ha = s.row(FD_H)[a];
    int count = 0;
    long long o = mode ? offs[tag] : 0;
    auto emit = [&](int b) {
        if (mode) idx[o + count] = s.irow(FI_TAG)[b];
        count++;
    };
    auto geom_ok = [&](int b, const int *sh, bool check_h) -> bool {
        double dx[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++)
            dx[d] = dsub(ra[d], image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]));
        const double r2 = exact_len2(dx, c.nd);
        if (check_h) {
            const double hb = s.row(FD_H)[b];
            const double t = 2.0 * (ha > hb ? ha : hb);
            if (r2 > dmul(t, t)) return false;
        }
        if ((sh[0] | sh[1] | sh[2]) && !image_exists(s.irow(FI_GCODE)[b], sh, c.nd)) return false;
        return true;
    };
    auto scan = [&](const CellCoord &cc, const int *dims, int base, auto &&body) {
        for (int ox = -1; ox <= 1; ox++)
            for (int oy = (c.nd > 1 ? -1 : 0); oy <= (c.nd > 1 ? 1 : 0); oy++)
                for (int oz = (c.nd > 2 ? -1 : 0); oz <= (c.nd > 2 ? 1 : 0); oz++) {
                    int sh[3];
                    const int lin = neighbour_cell(cc, ox, oy, oz, dims, c.periodic, c.nd, sh);
                    if (lin < 0) continue;
                    for (int b = start[base + lin]; b < start[base + lin + 1]; b++) body(b, sh);
                }
    };
    if (kind == SPHDEM_PAIRS_SPH && !dem) {
        scan(cell_sph(c, g, ra), g->sdims, 0, [&](int b, const int *sh) {
            if (b == a && !(sh[0] | sh[1] | sh[2])) return;
            if (geom_ok(b, sh, true)) emit(b);
        });
    } else if (kind == SPHDEM_PAIRS_DEM && dem) {
        scan(cell_dem(c, ra), c.ddims, g->n_sph_cells, [&](int b, const int *sh) {
            if (b == a && !(sh[0] | sh[1] | sh[2])) return;
            if (s.irow(FI_IAM)[b] != T_DEM) return;
            if (geom_ok(b, sh, true)) emit(b);
        });
    } else if (kind == SPHDEM_PAIRS_COUPLE_DS && dem) {
        scan(cell_sph(c, g, ra), g->sdims, 0, [&](int b, const int *sh) {
            if (geom_ok(b, sh, true)) emit(b);
        });
    } else if (kind == SPHDEM_PAIRS_COUPLE_SD && c.liq_dem() && is_sph_or_sphb(ta)) {
        int cs[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) cs[d] = ref_dem_cell(ra[d], c, d);
        scan(cell_dem(c, ra), c.ddims, g->n_sph_cells, [&](int b, const int *sh) {
            if (s.irow(FI_IAM)[b] != T_DEM) return;
            int cd[3] = {0, 0, 0};
            double dx[3] = {0, 0, 0};
            for (int d = 0; d < c.nd; d++) {
                const double rb = image_pos(s.row(FD_R + d)[b], sh[d], c.rmin[d], c.rmax[d]);
                cd[d] = ref_dem_cell(rb, c, d);
                dx[d] = dsub(ra[d], rb);
            }
            if (!coupling_rule(cs, cd, c)) return;
            if (!(exact_len2(dx, c.nd) < c.rc2)) return;
            if (!geom_ok(b, sh, false)) return;
            emit(b);
        });
    }
    if (!mode) cnt[tag] = count;
}

__global__ void k_cells(DevCfg c, DevState s, const DevGlobals *g, int64_t n, int *out) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int tag = s.irow(FI_TAG)[a];
    const int t = s.irow(FI_IAM)[a];
    for (int d = 0; d < 3; d++) {
        int v = 0;
        if (d < c.nd && t != T_DEAD) {
            const double r = s.row(FD_R + d)[a];
            v = (c.liq_dem() && t == T_DEM) ? ref_dem_cell(r, c, d)
                                            : trunc_index(r, c.dmin[d], g->sr2, g->rsr2_f, 3.0);
        }
        out[3 * (int64_t)tag + d] = v;
    }
}

}  // namespace

int export_pairs(sphdem_ctx *c, int kind, int64_t *offs, int32_t *idx, int64_t cap, int64_t *np) {
    const int64_t n = c->n;
    int *dcnt = nullptr;
    long long *doffs = nullptr;
    int *didx = nullptr;
    SPHDEM_CUDA_CHECK(cudaMalloc(&dcnt, n * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(dcnt, 0, n * sizeof(int), c->stream));
    /* mixed precision: sph/sphBoundary rows come from the FP32-built lists */
    const bool from_list = kind == SPHDEM_PAIRS_SPH && c->mx_maxn > 0;
    k_pairs<<<grid_for(n, BLK), BLK, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, n, kind, 0, dcnt, nullptr,
                                                     nullptr, (int)from_list);
    if (from_list) mixed_list_export(c, dcnt, nullptr, nullptr);
    std::vector<int> hcnt(n);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(hcnt.data(), dcnt, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    std::vector<long long> hoffs(n + 1, 0);
    for (int64_t i = 0; i < n; i++) hoffs[i + 1] = hoffs[i] + hcnt[i];
    *np = hoffs[n];
    if (offs)
        for (int64_t i = 0; i <= n; i++) offs[i] = hoffs[i];
    int rc = SPHDEM_OK;
    if (idx) {
        if (hoffs[n] > cap) {
            rc = SPHDEM_ERR_CAPACITY;
        } else if (hoffs[n] > 0) {
            SPHDEM_CUDA_CHECK(cudaMalloc(&doffs, (n + 1) * sizeof(long long)));
            SPHDEM_CUDA_CHECK(cudaMalloc(&didx, hoffs[n] * sizeof(int)));
            SPHDEM_CUDA_CHECK(cudaMemcpyAsync(doffs, hoffs.data(), (n + 1) * sizeof(long long),
                                              cudaMemcpyHostToDevice, c->stream));
            k_pairs<<<grid_for(n, BLK), BLK, 0, c->stream>>>(c->cfg, c->A, c->buf.start, c->g, n, kind, 1, dcnt,
                                                             doffs, didx, (int)from_list);
            if (from_list) mixed_list_export(c, dcnt, doffs, didx);
            SPHDEM_CUDA_CHECK(cudaMemcpyAsync(idx, didx, hoffs[n] * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
            for (int64_t i = 0; i < n; i++) std::sort(idx + hoffs[i], idx + hoffs[i + 1]);
        }
    }
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    cudaFree(dcnt);
    cudaFree(doffs);
    cudaFree(didx);
    return rc;
}

int export_cells(sphdem_ctx *c, int32_t *cells) {
    const int64_t n = c->n;
    int *d = nullptr;
    SPHDEM_CUDA_CHECK(cudaMalloc(&d, 3 * n * sizeof(int)));
    k_cells<<<grid_for(n, BLK), BLK, 0, c->stream>>>(c->cfg, c->A, c->g, n, d);
    SPHDEM_CUDA_CHECK(cudaMemcpyAsync(cells, d, 3 * n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHDEM_CUDA_CHECK(cudaStreamSynchronize(c->stream));
    SPHDEM_CUDA_CHECK(cudaGetLastError());
    cudaFree(d);
    return SPHDEM_OK;
}

/* ---------------------------------------------------------------------- */
/* Allocation-free bucket-index export.
 *
 * Same kernel and result as export_cells, but the 3n-int device staging
 * buffer is a fixed file-scope array instead of a cudaMalloc/cudaFree pair,
 * for callers that must not allocate device memory (a diagnostics hook that
 * runs after an out-of-memory failure, or a loop that cannot take the
 * device-wide synchronisation cudaFree implies).
 *
 * - Capacity: SPHDEM_CELL_IDS_NOALLOC_MAX particles (3 int32 each, 3 MiB of
 *   static device memory per device that loads this module); larger
 *   simulations are rejected with SPHDEM_ERR_CAPACITY.
 * - Every call looks the array's device address up with cudaGetSymbolAddress
 *   on the handle's device (cheap; the first call on a device can load the
 *   module there), so no address outlives a device reset.  Make the first
 *   call on a device before any stream capture on it.
 * - Every call on a device shares the one array: calls that overlap in time
 *   (from several threads, or several handles on one device) race on it.
 *   Nothing in it needs to start at zero: k_cells writes all 3n entries
 *   (tags are a permutation of 0..n-1) before the copy-out reads them.
 */
namespace {

static __device__ __align__(256) int32_t g_cells_scratch[3 * SPHDEM_CELL_IDS_NOALLOC_MAX];

}  // namespace

int export_cells_noalloc(sphdem_ctx *c, int32_t *cells) {
    const int64_t n = c->n;
    if (n > SPHDEM_CELL_IDS_NOALLOC_MAX) {
        c->err = "sphdem_cell_ids_noalloc: " + std::to_string(n) + " particles exceed the static buffer of " +
                 std::to_string(SPHDEM_CELL_IDS_NOALLOC_MAX) + " (use sphdem_cell_ids)";
        return SPHDEM_ERR_CAPACITY;
    }
    /* the handle's device: the one that owns its globals block */
    cudaPointerAttributes attr{};
    SPHDEM_CUDA_CHECK(cudaPointerGetAttributes(&attr, c->g));
    const int dev = attr.device;
    if (dev < 0) {
        c->err = "sphdem_cell_ids_noalloc: the handle's device could not be resolved";
        return SPHDEM_ERR_UNSUPPORTED;
    }
    int prev = -1;
    SPHDEM_CUDA_CHECK(cudaGetDevice(&prev));
    if (prev != dev) SPHDEM_CUDA_CHECK(cudaSetDevice(dev));
    /* the array's address on this device, looked up with the device current */
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_cells_scratch);
    int32_t *scratch = static_cast<int32_t *>(p);
    if (e == cudaSuccess && n > 0) {
        k_cells<<<grid_for(n, BLK), BLK, 0, c->stream>>>(c->cfg, c->A, c->g, n, scratch);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cells, scratch, 3 * n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    if (prev != dev) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        c->err = std::string("sphdem_cell_ids_noalloc: ") + cudaGetErrorString(e);
        return SPHDEM_ERR_CUDA;
    }
    return SPHDEM_OK;
}

}  // namespace sphdem
