/*
 * Rebuild of the bucket lists: the GPU form of CdataLL::reset
 * (dataLL.cpp:140-236) including the single-rank part of updateDomain
 * (dataLL.cpp:319-700).
 *
 *   k_migrate   periodic wrap / out-of-domain deletion (dataLL.cpp:371-404,
 *               464-516) and the next h_max (calcDomainLimits, 954-975)
 *   k_ghost     which periodic images exist (dataLL.cpp:522-582): the clipped
 *               inCoords of every particle, against the ghost widths
 *               procGhostMax2H of the previous rebuild (Rc for DEM), and the
 *               per-slot maximum h that sets the next widths (688-693)
 *   k_finalize  new widths, h_max, the search-radius hysteresis (220-223)
 *               and the SPH bucket grid size
 *   k_keys      bucket key of every particle: getCellI (dataLL.h:303-305) on
 *               non-periodic axes, an L/floor(L/2h) grid on periodic axes;
 *               DEM particles go to the DEM search grid
 *   k_scan_*    bucket starts
 *   k_scatter + k_rank   deterministic counting sort by bucket, and within
 *               a bucket by the coordinate on the last axis (ties by tag), so
 *               that a run of consecutive buckets along that axis is sorted
 *               by it and the slice passes can cut their candidate ranges
 *               by binary search
 *   k_gather    one launch moves every live field row into sorted order
 *
 * All sizes and widths live in DevGlobals, so the sequence replays in a CUDA
 * graph.  Roofline: HBM-bound; per particle it reads r (8d B) and writes a
 * key (4 B) twice, then the gather reads+writes every live row.
 */
#include "internal.cuh"

namespace sphdem {
namespace {

constexpr int BLK = 256;

__global__ void k_migrate(DevCfg c, DevState s, DevGlobals *g, unsigned char *mark, int64_t n) {
    __shared__ unsigned long long bmax;
    if (threadIdx.x == 0) bmax = 0ull;
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double h = -1.0;
    if (i < n) {
        int *iam = s.irow(FI_IAM);
        if (mark[i]) {
            /* markForDeletion (tag -111) is honoured first (dataLL.cpp:377-380) */
            mark[i] = 0;
            iam[i] = T_DEAD;
        }
        if (iam[i] != T_DEAD) {
            int oc[3] = {1, 1, 1};
            bool lost = false, out = false;
            for (int d = 0; d < c.nd; d++) {
                const double r = s.row(FD_R + d)[i];
                oc[d] = trunc_index(r, c.dmin[d], c.dspace[d], c.rdspace_f[d], 1.0);
                if (oc[d] > 2 || oc[d] < 0) lost = true;
                if (oc[d] != 1) {
                    out = true;
                    if (!c.periodic[d]) lost = true;
                }
            }
            if (lost) {
                iam[i] = T_DEAD;
                atomicAdd((unsigned long long *)&g->n_deleted, 1ull);
            } else {
                if (out) {
                    for (int d = 0; d < c.nd; d++) {
                        double *r = s.row(FD_R + d);
                        if (oc[d] == 2) r[i] = dadd(dsub(c.rmin[d], c.rmax[d]), r[i]);
                        else if (oc[d] == 0) r[i] = dadd(dsub(c.rmax[d], c.rmin[d]), r[i]);
                    }
                }
                h = s.row(FD_H)[i];
            }
        }
    }
    /* block maximum of h, then one atomic per block */
    for (int o = 16; o > 0; o >>= 1) h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
    if ((threadIdx.x & 31) == 0 && h >= 0.0) atomicMax(&bmax, dbits(h));
    __syncthreads();
    if (threadIdx.x == 0 && bmax) atomicMax(&g->hmax_bits, bmax);
}

__device__ __forceinline__ int slot_index(const int *co, int nd) {
    int sidx = 0;
    for (int i = 0; i < nd; i++) sidx = sidx * 3 + co[i];
    return sidx;
}

__global__ void k_ghost(DevCfg c, DevState s, DevGlobals *g, int64_t n) {
    __shared__ unsigned long long smax[27];
    if (threadIdx.x < 27) smax[threadIdx.x] = 0ull;
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) {
        const int t = s.irow(FI_IAM)[i];
        int gcode = 0;
        if (t != T_DEAD) {
            const bool dem = c.liq_dem() && t == T_DEM;
            int ic[3] = {1, 1, 1};
            bool any = false;
            for (int d = 0; d < c.nd; d++) {
                if (!c.periodic[d]) continue;
                const double r = s.row(FD_R + d)[i];
                int v = dem ? trunc_index(r, c.dg_lo[d], c.dg_sp[d], c.dg_rsp_f[d], 1.0)
                            : trunc_index(r, g->ghost_lo[d], g->ghost_sp[d], g->ghost_rsp_f[d], 1.0);
                if (v > 2) v = 2;
                if (v < 0) v = 0;
                ic[d] = v;
                any |= v != 1;
            }
            for (int d = 0; d < c.nd; d++) gcode |= ic[d] << (2 * d);
            if (any) {
                const double h = s.row(FD_H)[i];
                int lo3[3], hi3[3];
                for (int d = 0; d < 3; d++) {
                    lo3[d] = d < c.nd ? min(ic[d], 1) : 1;
                    hi3[d] = d < c.nd ? max(ic[d], 1) : 1;
                }
                for (int a = lo3[0]; a <= hi3[0]; a++)
                    for (int b = lo3[1]; b <= hi3[1]; b++)
                        for (int e = lo3[2]; e <= hi3[2]; e++) {
                            const int dc[3] = {a, b, e};
                            bool centre = true;
                            for (int d = 0; d < c.nd; d++) centre &= dc[d] == 1;
                            if (centre) continue;
                            int sl[3];
                            for (int d = 0; d < c.nd; d++) sl[d] = 2 - dc[d];
                            atomicMax(&smax[slot_index(sl, c.nd)], dbits(h));
                        }
            }
        }
        s.irow(FI_GCODE)[i] = gcode;
    }
    __syncthreads();
    if (threadIdx.x < 27 && smax[threadIdx.x]) atomicMax(&g->slot_bits[threadIdx.x], smax[threadIdx.x]);
}

__global__ void k_finalize(DevCfg c, DevGlobals *g) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    bool any_periodic = false;
    for (int d = 0; d < c.nd; d++) any_periodic |= c.periodic[d] != 0;
    const int ns = c.nd == 3 ? 27 : (c.nd == 2 ? 9 : 3);
    if (any_periodic) {
        for (int sidx = 0; sidx < ns; sidx++) {
            int co[3], t = sidx;
            for (int d = c.nd - 1; d >= 0; d--) {
                co[d] = t % 3;
                t /= 3;
            }
            bool centre = true, has = true;
            for (int d = 0; d < c.nd; d++)
                if (co[d] != 1) {
                    centre = false;
                    if (!c.periodic[d]) has = false;
                }
            if (centre || !has) continue;
            const double smax = __longlong_as_double((long long)g->slot_bits[sidx]);
            const double maxh = smax > g->hmax ? smax : g->hmax;
            g->gw[sidx] = 2.0 * maxh;
        }
    }
    const double hmax = __longlong_as_double((long long)g->hmax_bits);
    g->hmax = hmax;
    for (int d = 0; d < c.nd; d++) {
        for (int side = 0; side <= 2; side += 2) {
            int co[3] = {1, 1, 1};
            co[d] = side;
            int sidx = 0;
            for (int k = 0; k < c.nd; k++) sidx = sidx * 3 + co[k];
            if (g->gw[sidx] < hmax) g->gw[sidx] = 2.0 * hmax;
        }
    }
    if (hmax > g->sr || hmax < 0.9 * g->sr) g->sr = hmax;
    g->sr2 = 2.0 * g->sr;
    g->rsr2_f = (float)(1.0 / g->sr2);
    /* SPH ghost test of the next rebuild (dataLL.cpp:338-364) */
    for (int d = 0; d < c.nd; d++) {
        int co[3] = {1, 1, 1};
        co[d] = 0;
        int slo = 0, shi = 0;
        for (int k = 0; k < c.nd; k++) slo = slo * 3 + co[k];
        co[d] = 2;
        for (int k = 0; k < c.nd; k++) shi = shi * 3 + co[k];
        g->ghost_lo[d] = c.dmin[d] + g->gw[slo];
        double sp = c.dspace[d] - g->gw[slo];
        sp -= g->gw[shi];
        g->ghost_sp[d] = sp;
        g->ghost_rsp_f[d] = (float)(1.0 / sp);
    }
    int tot = 1;
    for (int d = 0; d < 3; d++) {
        if (d >= c.nd) {
            g->sdims[d] = 1;
            g->scell[d] = 1.0;
            continue;
        }
        const double ext = c.dmax[d] - c.dmin[d];
        if (c.periodic[d]) {
            int m = (int)floor(ext / (2.0 * g->sr * (1.0 + 1e-12)));
            if (m < 3) {
                set_err(g, SPHDEM_ERR_CAPACITY, 100 + d);
                m = 3;
            }
            g->sdims[d] = m;
            g->scell[d] = ext / m;
            g->rscell[d] = m / ext;
        } else {
            g->sdims[d] = (int)(ext / (2.0 * g->sr)) + 8;
            g->scell[d] = 2.0 * g->sr;
        }
        tot *= g->sdims[d];
    }
    if (tot > c.sph_cells_cap) {
        set_err(g, SPHDEM_ERR_CAPACITY, tot);
        tot = c.sph_cells_cap;
    }
    g->n_sph_cells = tot;
    g->n_total_cells = tot + c.n_dem_cells + 1;
    g->hmax_bits = 0ull;
    for (int k = 0; k < 27; k++) g->slot_bits[k] = 0ull;
}

__device__ __forceinline__ int dem_grid_cell(const DevCfg &c, const double *r, int *cc) {
    int lin = 0;
    for (int d = 0; d < c.nd; d++) {
        int k = (int)floor((r[d] - c.dorig[d]) * c.rdcell[d]);
        if (k < 0) k = c.periodic[d] ? c.ddims[d] - 1 : 0;
        if (k >= c.ddims[d]) k = c.periodic[d] ? 0 : c.ddims[d] - 1;
        cc[d] = k;
        lin = lin * c.ddims[d] + k;
    }
    return lin;
}

__global__ void k_keys(DevCfg c, DevState s, DevGlobals *g, int *key, int *cnt, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s.irow(FI_IAM)[i];
    int k;
    if (t == T_DEAD) {
        k = g->n_total_cells - 1;
    } else {
        double r[3] = {0, 0, 0};
        for (int d = 0; d < c.nd; d++) r[d] = s.row(FD_R + d)[i];
        if (c.liq_dem() && t == T_DEM) {
            int cc[3];
            k = g->n_sph_cells + dem_grid_cell(c, r, cc);
            for (int d = 0; d < 3; d++) s.irow(FI_RDC0 + d)[i] = d < c.nd ? ref_dem_cell(r[d], c, d) : 0;
        } else {
            int lin = 0;
            bool bad = false;
            for (int d = 0; d < c.nd; d++) {
                int ci;
                if (c.periodic[d]) {
                    ci = (int)floor((r[d] - c.dmin[d]) * g->rscell[d]);
                    if (ci < 0) ci = 0;
                    if (ci >= g->sdims[d]) ci = g->sdims[d] - 1;
                } else {
                    ci = trunc_index(r[d], c.dmin[d], g->sr2, g->rsr2_f, 3.0);
                    if (ci < 0 || ci >= g->sdims[d]) {
                        bad = true;
                        ci = 0;
                    }
                }
                lin = lin * g->sdims[d] + ci;
            }
            if (bad || lin >= g->n_sph_cells) {
                set_err(g, SPHDEM_ERR_OUT_OF_RANGE, (int)i);
                lin = 0;
            }
            k = lin;
        }
    }
    key[i] = k;
    atomicAdd(&cnt[k], 1);
}

/* three-phase exclusive scan of cnt[0..m) into start[0..m], start[m] = total */
constexpr int SCAN_BLK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLK * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const int before = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    return before + x - v;
}

__global__ void k_scan_reduce(const int *cnt, const DevGlobals *g, int *bsum) {
    __shared__ int ws[32];
    const int m = g->n_total_cells;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int acc = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int64_t j = base + threadIdx.x * SCAN_ITEMS + k;
        if (j < m) acc += cnt[j];
    }
    int total;
    block_exclusive_scan(acc, ws, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_blocks(int *bsum, int nblocks) {
    __shared__ int ws[32];
    int carry = 0;
    for (int base = 0; base < nblocks; base += blockDim.x) {
        const int j = base + threadIdx.x;
        const int v = j < nblocks ? bsum[j] : 0;
        int total;
        const int ex = block_exclusive_scan(v, ws, &total);
        __syncthreads();
        if (j < nblocks) bsum[j] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

__global__ void k_scan_down(const int *cnt, const DevGlobals *g, const int *bsum, int *start, int *fill) {
    __shared__ int ws[32];
    const int m = g->n_total_cells;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int v[SCAN_ITEMS];
    int acc = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int64_t j = base + threadIdx.x * SCAN_ITEMS + k;
        v[k] = j < m ? cnt[j] : 0;
        acc += v[k];
    }
    int run = block_exclusive_scan(acc, ws, nullptr) + bsum[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int64_t j = base + threadIdx.x * SCAN_ITEMS + k;
        if (j < m) {
            start[j] = run;
            fill[j] = 0;
        } else if (j == m) {
            start[j] = run;
        }
        run += v[k];
    }
    /* the end sentinel when m sits exactly at the end of this thread's items */
    if (base + (int64_t)(threadIdx.x + 1) * SCAN_ITEMS == m) start[m] = run;
}

/* order-preserving integer image of a double (integer compares are full rate) */
__device__ __forceinline__ unsigned long long order_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_scatter(const int *key, const int *start, int *fill, int *slot, const int *tag, const double *rz,
                          int *slot_tag, unsigned long long *slot_z, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = key[i];
    const int pos = start[k] + atomicAdd(&fill[k], 1);
    slot[pos] = (int)i;
    slot_tag[pos] = tag[i];
    slot_z[pos] = order_key(rz[i]);
}

/* rank within the bucket by (last-axis coordinate, tag) from the scatter's
 * contiguous copies: perm[start + rank] = previous slot */
__global__ void k_rank(const int *key, const int *start, const int *slot, const int *slot_tag,
                       const unsigned long long *slot_z, int *perm, int *skey, const DevGlobals *g, int64_t n) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int dead_key = g->n_total_cells - 1;
    const int i = slot[j];
    const int k = key[i];
    const int s0 = start[k], s1 = start[k + 1];
    int rank = (int)j - s0;  /* deleted particles: any order */
    if (k != dead_key) {
        const int my = slot_tag[j];
        const unsigned long long mz = slot_z[j];
        rank = 0;
        for (int u = s0; u < s1; u++) {
            const unsigned long long z = slot_z[u];
            rank += z < mz || (z == mz && slot_tag[u] < my);
        }
    }
    perm[s0 + rank] = i;
    skey[s0 + rank] = k;
}

/* one thread per particle and a group of rows (blockIdx.y): the permutation
 * is read once per group, and the group's loads are all in flight together */
constexpr int GATHER_ROWS = 8;
__global__ void k_gather(DevState src, DevState dst, const int *perm, const int *fd, int nfd,
                         const int *fi, int nfi, int64_t n) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    int p = perm[k];
    if (p < 0 || p >= n) p = 0;  /* never out of bounds, whatever the sort left */
    const int f0 = blockIdx.y * GATHER_ROWS;
    double v[GATHER_ROWS];
    int iv[GATHER_ROWS];
#pragma unroll
    for (int q = 0; q < GATHER_ROWS; q++) {
        const int f = f0 + q;
        if (f < nfd) v[q] = src.row(fd[f])[p];
        else if (f - nfd < nfi) iv[q] = src.irow(fi[f - nfd])[p];
    }
#pragma unroll
    for (int q = 0; q < GATHER_ROWS; q++) {
        const int f = f0 + q;
        if (f < nfd) dst.row(fd[f])[k] = v[q];
        else if (f - nfd < nfi) dst.irow(fi[f - nfd])[k] = iv[q];
    }
}

}  // namespace

void setup_rebuild_buffers(sphdem_ctx *c) {
    /* FP64 rows worth gathering: drop z components in 2D, coupling rows
     * without LIQ_DEM, normals when no repulsive boundary particle exists. */
    std::vector<int> fd, fi;
    const int nd = c->cfg.nd;
    const bool liq = c->cfg.liq_dem();
    auto vec = [&](int base) {
        for (int d = 0; d < nd; d++) fd.push_back(base + d);
    };
    vec(FD_R); vec(FD_V); vec(FD_VHAT); vec(FD_V0); vec(FD_VHAT0);
    vec(FD_F); vec(FD_FP); vec(FD_FV); vec(FD_FB);
    if (liq) { vec(FD_FDRAG); vec(FD_FVEL); vec(FD_GPOR); }
    vec(FD_N1); vec(FD_N2); if (nd == 3) vec(FD_N3);
    for (int f : {FD_MASS, FD_DENS, FD_DDDT, FD_H, FD_PRESS, FD_PDR2, FD_OMEGA, FD_RADIUS,
                  FD_IH, FD_IHN, FD_IHN2, FD_U, FD_DUDT, FD_EVISCF, FD_DEVISCF})
        fd.push_back(f);
    fd.push_back(FD_POR);
    if (liq) for (int f : {FD_DPORDT, FD_SHEP}) fd.push_back(f);
    fi = {FI_IAM, FI_TAG, FI_CONCAVE, FI_GCODE};
    if (liq) for (int f : {FI_RDC0, FI_RDC1, FI_RDC2}) fi.push_back(f);
    SPHDEM_CUDA_CHECK(cudaMalloc(&c->buf.fields_d, fd.size() * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMalloc(&c->buf.fields_i, fi.size() * sizeof(int)));
    SPHDEM_CUDA_CHECK(cudaMemcpy(c->buf.fields_d, fd.data(), fd.size() * sizeof(int), cudaMemcpyHostToDevice));
    SPHDEM_CUDA_CHECK(cudaMemcpy(c->buf.fields_i, fi.data(), fi.size() * sizeof(int), cudaMemcpyHostToDevice));
    c->buf.n_fields_d = (int)fd.size();
    c->buf.n_fields_i = (int)fi.size();
}

void rebuild(sphdem_ctx *c) {
    const int64_t n = c->n;
    const int gb = grid_for(n, BLK);
    Buffers &b = c->buf;
    SPHDEM_LAUNCH(c, "rebuild_migrate", k_migrate, gb, BLK, 0, c->cfg, c->A, c->g, c->delmark, n);
    SPHDEM_LAUNCH(c, "rebuild_ghost", k_ghost, gb, BLK, 0, c->cfg, c->A, c->g, n);
    SPHDEM_LAUNCH(c, "rebuild_finalize", k_finalize, 1, 32, 0, c->cfg, c->g);
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(b.cnt, 0, (size_t)b.cells_cap * sizeof(int), c->stream));
    SPHDEM_LAUNCH(c, "rebuild_keys", k_keys, gb, BLK, 0, c->cfg, c->A, c->g, b.key, b.cnt, n);
    const int nscan = (b.cells_cap + SCAN_TILE - 1) / SCAN_TILE;
    SPHDEM_LAUNCH(c, "rebuild_scan_reduce", k_scan_reduce, nscan, SCAN_BLK, 0, b.cnt, c->g, b.bsum);
    SPHDEM_LAUNCH(c, "rebuild_scan_blocks", k_scan_blocks, 1, SCAN_BLK, 0, b.bsum, nscan);
    SPHDEM_LAUNCH(c, "rebuild_scan_down", k_scan_down, nscan, SCAN_BLK, 0, b.cnt, c->g, b.bsum, b.start, b.fill);
    SPHDEM_CUDA_CHECK(cudaMemsetAsync(b.perm, 0, (size_t)n * sizeof(int), c->stream));
    SPHDEM_LAUNCH(c, "rebuild_scatter", k_scatter, gb, BLK, 0, b.key, b.start, b.fill, b.slot, c->A.irow(FI_TAG),
                  c->A.row(FD_R + c->cfg.nd - 1), b.slot_tag, b.slot_z, n);
    SPHDEM_LAUNCH(c, "rebuild_rank", k_rank, gb, BLK, 0, b.key, b.start, b.slot, b.slot_tag, b.slot_z, b.perm,
                  b.skey, c->g, n);
    dim3 gg(gb, (b.n_fields_d + b.n_fields_i + GATHER_ROWS - 1) / GATHER_ROWS);
    SPHDEM_LAUNCH(c, "rebuild_gather", k_gather, gg, BLK, 0, c->A, c->B, b.perm, b.fields_d,
                  b.n_fields_d, b.fields_i, b.n_fields_i, n);
    std::swap(c->A, c->B);
    c->flipped = !c->flipped;
}

}  // namespace sphdem
