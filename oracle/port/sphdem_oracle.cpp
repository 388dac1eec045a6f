/*
 * CPU oracle: a restatement, in plain C++, of the reference's per-step hot
 * path (martinjrobins/SPH-DEM).  TEST INFRASTRUCTURE ONLY -- the tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the
 * checker; the product path never links or calls it.
 *
 * Parity pin: tests/test_oracle_golden.py checks this port against golden
 * outputs of the reference itself (tests/golden/, produced by
 * tests/golden/make_golden.py from the unmodified reference sources built by
 * oracle/ref/build_ref.py).
 *
 * Structure follows the reference on purpose, so that its cost profile is
 * representative as a CPU baseline: an array of particle records (particle.h
 * Cparticle), bucket grids with the reference's index maps (dataLL.h:303-311),
 * ghost images for periodic axes (dataLL.cpp:319-700), per-particle cached
 * neighbour lists rebuilt at every reset (dataLL.cpp:1026-1075), the
 * uncached, asymmetric coupling search (dataLL.cpp:1104-1192) and the
 * start/middle/end sequence of sphIncompress.cpp:3-251.  Arithmetic follows
 * the reference expression by expression (pow, blitz's right-nested dot).
 *
 * Build: g++ -O2 -ffp-contract=off -shared -fPIC (oracle/build_oracle.py).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/sphdem.h"

namespace {

enum { T_SPH = 0, T_SPHB = 1, T_BOUNDARY = 3, T_BOBJ1 = 5, T_BOBJ6 = 10, T_DEM = 11 };

struct V3 {
    double x[3];
};

struct Part {
    int iam, tag;
    bool concave, alive;
    bool marked;           /* markForDeletion (tag -111): removed by the next reset */
    double r[3], v[3], vhat[3], v0[3], vhat0[3];
    double f[3], fp[3], fv[3], fb[3], ff[3];
    double fdrag[3], fvel[3], gradPor[3];
    double norm1[3], norm2[3], norm3[3];
    double mass, dens, dddt, h, press, pdr2, omega, porosity, dpordt, shep, radius;
    double u, dudt, eViscF, deViscFdt;   /* calcEnergies integrals (sphIncompress.h:769-781) */
    double invM[9], sumGrad[3], sum;     /* CORRECTED_GRADIENT (particle.h:243-246) */
};

/* A bucket entry: particle index plus the periodic image it stands for. */
struct Entry {
    int idx;
    int8_t s[3];
};

struct Sim {
    SphDemConfig c;
    int nd;
    std::vector<Part> ps;
    double time = 0, dt = 0, newDt = 0, maxdt = 0, demDt = 0;
    long long step = 0, n_deleted = 0;

    /* SPH bucket grid (dataLL.h:303-305), DEM bucket grid (dataLL.h:308-311) */
    double sph_sr;
    int sdim[3], ddim[3];
    std::vector<std::vector<Entry>> scells, dcells;
    std::vector<Entry> ghosts;
    std::vector<std::vector<Entry>> nbrs;  /* cached calcNeighbours lists */
    std::vector<int> order;                 /* container (ps) order        */
    std::vector<double> gw;                 /* procGhostMax2H per slot     */
    double hmax;                            /* CdataLL::hmax               */

    double wcon, L[3];

    /* ---------------- math, sph.h:29-342 ---------------- */
    static double dot(const double *a, const double *b, int nd) {
        /* blitz _bz_meta_vectorDot: a0*b0 + (a1*b1 + (a2*b2)) */
        if (nd == 3) return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
        if (nd == 2) return a[0] * b[0] + a[1] * b[1];
        return a[0] * b[0];
    }
    double len2(const double *a) const { return dot(a, a, nd); }
    double len(const double *a) const { return std::sqrt(len2(a)); }
    double K(double q) const { return q <= 2.0 ? wcon * std::pow(2.0 - q, 4) * (1.0 + 2.0 * q) : 0.0; }
    double Wk(double q, double h) const { return (1 / std::pow(h, nd)) * K(q); }
    double F(double q, double h) const {
        if (q <= 2.0)
            return (1 / std::pow(h, nd + 2)) * wcon *
                   (-4 * std::pow(2 - q, 3) * (1 + 2 * q) + 2 * std::pow(2 - q, 4)) / q;
        return 0.0;
    }
    double pdKh(double q, double h) const {
        if (q <= 2.0) return -wcon * q * (-4 * std::pow(2 - q, 3) * (1 + 2 * q) + 2 * std::pow(2 - q, 4)) / h;
        return 0.0;
    }
    double pdWh(double q, double h) const {
        return (1 / std::pow(h, nd)) * pdKh(q, h) - nd / std::pow(h, nd + 1) * K(q);
    }
    bool var_h() const { return c.flags & SPHDEM_F_VAR_H_CORRECTION; }
    bool liq_dem() const { return c.flags & SPHDEM_F_LIQ_DEM; }
    bool corrected() const { return c.flags & SPHDEM_F_CORRECTED_GRADIENT; }
    /* gradW, sph.h:322-342; with CORRECTED_GRADIENT the product
     * invM_a ((dr F - sumGrad_a/sum_a)/sum_a) (vect.h:39-47 row by row) */
    void gradW(const Part &pa, const double *dr, double q, double h, double *out) const {
        double drF[3] = {0, 0, 0};
        if (q != 0) {
            const double fq = F(q, h);
            for (int i = 0; i < nd; i++) drF[i] = dr[i] * fq;
        }
        double ret[3] = {0, 0, 0};
        if (corrected()) {
            double t[3] = {0, 0, 0};
            for (int i = 0; i < nd; i++) t[i] = (drF[i] - pa.sumGrad[i] / pa.sum) / pa.sum;
            for (int i = 0; i < nd; i++) {
                ret[i] = 0.0;
                for (int j = 0; j < nd; j++) ret[i] += pa.invM[i * nd + j] * t[j];
            }
        } else {
            for (int i = 0; i < nd; i++) ret[i] = drF[i];
        }
        for (int i = 0; i < nd; i++) out[i] = var_h() ? ret[i] / pa.omega : ret[i];
    }
    static bool is_boundary(int t) { return t == T_BOUNDARY || (t >= T_BOBJ1 && t <= T_BOBJ6); }

    /* entry position (ghost images shifted by the periodic extent) */
    void epos(const Entry &e, double *out) const {
        const Part &p = ps[e.idx];
        for (int i = 0; i < nd; i++) out[i] = e.s[i] == 0 ? p.r[i] : (e.s[i] > 0 ? (c.rmax[i] - c.rmin[i]) + p.r[i] : (c.rmin[i] - c.rmax[i]) + p.r[i]);
    }

    /* ---------------- grids ---------------- */
    void sph_cell(const double *r, int *ci) const {
        for (int i = 0; i < nd; i++) ci[i] = (int)((r[i] - c.domain_min[i]) / (2.0 * sph_sr) + 3);
    }
    void dem_cell(const double *r, int *ci) const {
        for (int i = 0; i < nd; i++)
            ci[i] = (int)((r[i] - c.domain_min[i]) / (2 * c.dem_search_radius) +
                          2 * c.coupling_radius / c.dem_search_radius - 1);
    }
    long long lin(const int *ci, const int *dims) const {
        long long l = 0;
        for (int i = 0; i < nd; i++) {
            if (ci[i] < 0 || ci[i] >= dims[i]) return -1;
            l = l * dims[i] + ci[i];
        }
        return l;
    }

    void resize_sph_grid() {
        long long tot = 1;
        for (int i = 0; i < nd; i++) {
            sdim[i] = (int)((c.domain_max[i] - c.domain_min[i]) / (2.0 * sph_sr)) + 8;
            tot *= sdim[i];
        }
        scells.assign(tot, std::vector<Entry>());
    }
    void init_grids() {
        sph_sr = c.h;
        resize_sph_grid();
        if (liq_dem()) {
            long long tot = 1;
            for (int i = 0; i < nd; i++) {
                ddim[i] = (int)((c.domain_max[i] - c.domain_min[i]) / (2 * c.dem_search_radius) +
                                2 * 2 * c.coupling_radius / c.dem_search_radius);
                tot *= ddim[i];
            }
            dcells.assign(tot, std::vector<Entry>());
        }
        gw.assign(nslots(), 1.1 * 2.0 * c.h);
        hmax = c.h;
        order.resize(ps.size());
        for (size_t k = 0; k < ps.size(); k++) order[k] = (int)k;
    }

    void insert(const Entry &e) {
        double r[3];
        epos(e, r);
        int ci[3];
        if (liq_dem() && ps[e.idx].iam == T_DEM) {
            dem_cell(r, ci);
            long long l = lin(ci, ddim);
            if (l < 0) throw std::string("DEM particle outside the bucket grid");
            dcells[l].push_back(e);
        } else {
            sph_cell(r, ci);
            long long l = lin(ci, sdim);
            if (l < 0) throw std::string("particle outside the bucket grid");
            scells[l].push_back(e);
        }
    }

    /* ---- single-rank updateDomain bookkeeping (dataLL.cpp:319-700) ----
     * slots are the 3^nd neighbour directions, row-major (blitz storage
     * order); a slot has a neighbour iff every non-centre axis is periodic. */
    int nslots() const { return nd == 3 ? 27 : nd == 2 ? 9 : 3; }
    void slot_coords(int s, int *co) const {
        for (int i = nd - 1; i >= 0; i--) { co[i] = s % 3; s /= 3; }
    }
    int slot_index(const int *co) const {
        int s = 0;
        for (int i = 0; i < nd; i++) s = s * 3 + co[i];
        return s;
    }
    bool slot_has_neighbour(const int *co) const {
        bool centre = true;
        for (int i = 0; i < nd; i++)
            if (co[i] != 1) {
                centre = false;
                if (!c.periodic[i]) return false;
            }
        return !centre;
    }
    int face_slot(int dim, int side) const {
        int co[3] = {1, 1, 1};
        co[dim] = side;
        return slot_index(co);
    }

    /* CdataLL::reset, dataLL.cpp:140-236, with updateDomain's single-rank
     * semantics: migration with periodic wrap or deletion (371-516), ghost
     * images within procGhostMax2H of a periodic face (522-695), then
     * calcDomainLimits (954-975), the search-radius hysteresis (220-223) and
     * insertion of particles in container order followed by the ghosts. */
    void reset() {
        for (auto &v : scells) v.clear();
        for (auto &v : dcells) v.clear();
        ghosts.clear();
        const int ns = nslots();
        /* migration */
        std::vector<std::vector<int>> recv(ns);
        for (size_t pos = 0; pos < order.size();) {
            const int k = order[pos];
            Part &p = ps[k];
            if (p.marked) {
                /* updateDomain deletes tag -111 first (dataLL.cpp:377-380) */
                p.alive = false;
                p.marked = false;
                order[pos] = order.back();
                order.pop_back();
                continue;
            }
            int oc[3] = {1, 1, 1};
            bool lost = false, out = false;
            for (int i = 0; i < nd; i++) {
                const double dspace = c.domain_max[i] - c.domain_min[i];
                oc[i] = (int)((p.r[i] - c.domain_min[i]) / dspace + 1);
                if (oc[i] > 2 || oc[i] < 0) lost = true;
                if (oc[i] != 1) out = true;
            }
            if (!lost && out) {
                if (slot_has_neighbour(oc)) {
                    int sl[3] = {1, 1, 1};
                    for (int i = 0; i < nd; i++) sl[i] = 2 - oc[i];
                    recv[slot_index(sl)].push_back(k);
                } else {
                    lost = true;
                }
            }
            if (lost) {
                p.alive = false;
                n_deleted++;
            }
            if (lost || out) {
                order[pos] = order.back();
                order.pop_back();
                continue;
            }
            pos++;
        }
        for (int s = 0; s < ns; s++) {
            int sl[3] = {1, 1, 1};
            slot_coords(s, sl);
            for (int k : recv[s]) {
                Part &p = ps[k];
                for (int i = 0; i < nd; i++) {
                    if (c.periodic[i] && sl[i] == 0) p.r[i] = c.rmin[i] - c.rmax[i] + p.r[i];
                    if (c.periodic[i] && sl[i] == 2) p.r[i] = c.rmax[i] - c.rmin[i] + p.r[i];
                }
                order.push_back(k);
            }
        }
        /* ghosts */
        bool any_periodic = false;
        for (int i = 0; i < nd; i++) any_periodic |= c.periodic[i] != 0;
        if (any_periodic) {
            double dgmin[3], dgspace[3], ddmin[3], ddspace[3];
            for (int i = 0; i < nd; i++) {
                const double dspace = c.domain_max[i] - c.domain_min[i];
                const double lo = gw[face_slot(i, 0)], hi = gw[face_slot(i, 2)];
                dgmin[i] = c.domain_min[i] + lo;
                dgspace[i] = dspace - lo;
                dgspace[i] -= hi;
                ddmin[i] = c.domain_min[i] + c.coupling_radius;
                ddspace[i] = dspace - c.coupling_radius;
                ddspace[i] -= c.coupling_radius;
            }
            std::vector<std::vector<int>> gsend(ns);
            for (int k : order) {
                const Part &p = ps[k];
                const bool dem = liq_dem() && p.iam == T_DEM;
                int ic[3] = {1, 1, 1}, lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
                bool any = false;
                for (int i = 0; i < nd; i++) {
                    ic[i] = dem ? (int)((p.r[i] - ddmin[i]) / ddspace[i] + 1)
                                : (int)((p.r[i] - dgmin[i]) / dgspace[i] + 1);
                    if (ic[i] > 2) ic[i] = 2;
                    if (ic[i] < 0) ic[i] = 0;
                    if (ic[i] != 1) any = true;
                    lo[i] = ic[i] <= 1 ? ic[i] : 1;
                    hi[i] = ic[i] <= 1 ? 1 : ic[i];
                }
                if (!any) continue;
                int d[3] = {1, 1, 1};
                for (d[0] = lo[0]; d[0] <= hi[0]; d[0]++)
                    for (d[1] = (nd > 1 ? lo[1] : 1); d[1] <= (nd > 1 ? hi[1] : 1); d[1]++)
                        for (d[2] = (nd > 2 ? lo[2] : 1); d[2] <= (nd > 2 ? hi[2] : 1); d[2]++) {
                            if (!slot_has_neighbour(d)) continue;
                            int sl[3] = {1, 1, 1};
                            for (int i = 0; i < nd; i++) sl[i] = 2 - d[i];
                            gsend[slot_index(sl)].push_back(k);
                        }
            }
            for (int s = 0; s < ns; s++) {
                int sl[3] = {1, 1, 1};
                slot_coords(s, sl);
                if (!slot_has_neighbour(sl)) continue;
                double maxh = hmax;
                for (int k : gsend[s]) {
                    Entry e{k, {0, 0, 0}};
                    for (int i = 0; i < nd; i++) e.s[i] = sl[i] == 0 ? -1 : (sl[i] == 2 ? 1 : 0);
                    ghosts.push_back(e);
                    if (ps[k].h > maxh) maxh = ps[k].h;
                }
                gw[s] = 2.0 * maxh;
            }
        }
        /* calcDomainLimits */
        hmax = -100000;
        for (int k : order)
            if (ps[k].h > hmax) hmax = ps[k].h;
        for (int i = 0; i < nd; i++) {
            for (int side = 0; side <= 2; side += 2) {
                double &g = gw[face_slot(i, side)];
                if (g < hmax) g = 2.0 * hmax;
            }
        }
        if (hmax > sph_sr || hmax < 0.9 * sph_sr) {
            sph_sr = hmax;
            resize_sph_grid();
        }
        for (int k : order) insert(Entry{k, {0, 0, 0}});
        for (const Entry &e : ghosts) insert(e);
        /* neighbour lists for every real particle (the reference builds them
         * lazily on first use after the reset, at the same positions) */
        const int n = ps.size();
        nbrs.assign(n, std::vector<Entry>());
        for (int k : order) calc_neighbours(k, nbrs[k]);
    }

    /* CdataLL::calcNeighbours, dataLL.cpp:1026-1075 with is_neighbr,
     * particle.h:236-238 */
    void calc_neighbours(int k, std::vector<Entry> &out) const {
        const Part &p = ps[k];
        int ci[3];
        const bool dem = liq_dem() && p.iam == T_DEM;
        if (dem) dem_cell(p.r, ci); else sph_cell(p.r, ci);
        const int *dims = dem ? ddim : sdim;
        const auto &cells = dem ? dcells : scells;
        int t[3] = {0, 0, 0};
        for (t[0] = ci[0] - 1; t[0] <= ci[0] + 1; t[0]++)
            for (t[1] = (nd > 1 ? ci[1] - 1 : 0); t[1] <= (nd > 1 ? ci[1] + 1 : 0); t[1]++)
                for (t[2] = (nd > 2 ? ci[2] - 1 : 0); t[2] <= (nd > 2 ? ci[2] + 1 : 0); t[2]++) {
                    long long l = lin(t, dims);
                    if (l < 0) continue;
                    for (const Entry &e : cells[l]) {
                        if (e.idx == k && e.s[0] == 0 && e.s[1] == 0 && e.s[2] == 0) continue;
                        double rb[3], d[3];
                        epos(e, rb);
                        for (int i = 0; i < nd; i++) d[i] = p.r[i] - rb[i];
                        const double hm = std::max(p.h, ps[e.idx].h);
                        const double rad = 2.0 * hm;
                        if (len2(d) <= rad * rad) out.push_back(e);
                    }
                }
    }

    /* CdataLL::calcNeighboursCoupling, dataLL.cpp:1104-1192 */
    void calc_coupling(int k, std::vector<Entry> &out) const {
        const Part &p = ps[k];
        int ci[3], t[3] = {0, 0, 0};
        if (p.iam == T_DEM) {
            sph_cell(p.r, ci);
            for (t[0] = ci[0] - 1; t[0] <= ci[0] + 1; t[0]++)
                for (t[1] = (nd > 1 ? ci[1] - 1 : 0); t[1] <= (nd > 1 ? ci[1] + 1 : 0); t[1]++)
                    for (t[2] = (nd > 2 ? ci[2] - 1 : 0); t[2] <= (nd > 2 ? ci[2] + 1 : 0); t[2]++) {
                        long long l = lin(t, sdim);
                        if (l < 0) continue;
                        for (const Entry &e : scells[l]) {
                            double rb[3], d[3];
                            epos(e, rb);
                            for (int i = 0; i < nd; i++) d[i] = p.r[i] - rb[i];
                            const double rad = 2.0 * std::max(p.h, ps[e.idx].h);
                            if (len2(d) <= rad * rad) out.push_back(e);
                        }
                    }
            return;
        }
        const int num = (int)std::ceil(0.5 * c.coupling_radius / c.dem_search_radius);
        const double lim = std::pow(0.5 * c.coupling_radius / c.dem_search_radius, 2);
        const double rc2 = std::pow(c.coupling_radius, 2);
        dem_cell(p.r, ci);
        for (t[0] = ci[0] - num; t[0] <= ci[0] + num; t[0]++) {
            const int iP = (t[0] - ci[0] + 1) * (t[0] - ci[0] + 1);
            const int iM = (t[0] - ci[0] - 1) * (t[0] - ci[0] - 1);
            for (t[1] = (nd > 1 ? ci[1] - num : 0); t[1] <= (nd > 1 ? ci[1] + num : 0); t[1]++) {
                const int jP = nd > 1 ? (t[1] + 1 - ci[1]) * (t[1] + 1 - ci[1]) : 0;
                const int jM = nd > 1 ? (t[1] - 1 - ci[1]) * (t[1] - 1 - ci[1]) : 0;
                for (t[2] = (nd > 2 ? ci[2] - num : 0); t[2] <= (nd > 2 ? ci[2] + num : 0); t[2]++) {
                    int rP, rM;
                    if (nd > 2) {
                        rP = iP + jP + (t[2] - ci[2] + 1) * (t[2] - ci[2] + 1);
                        rM = iM + jM + (t[2] - ci[2] - 1) * (t[2] - ci[2] - 1);
                    } else {
                        rP = iP + jP;
                        rM = iM + jM;
                    }
                    const bool all = nd > 1 && rP < lim;
                    const bool some = nd == 1 || (!all && rM < lim);
                    if (!all && !some) continue;
                    long long l = lin(t, ddim);
                    if (l < 0) continue;
                    for (const Entry &e : dcells[l]) {
                        if (all) {
                            out.push_back(e);
                        } else {
                            double rb[3], d[3];
                            epos(e, rb);
                            for (int i = 0; i < nd; i++) d[i] = p.r[i] - rb[i];
                            if (len2(d) < rc2) out.push_back(e);
                        }
                    }
                }
            }
        }
    }

    /* ---------------- integrators, sphIncompress.h:620-767 ---------------- */
    static bool sph_or_sphb(int t) { return t == T_SPH || t == T_SPHB; }

    void drift_r(Part &p, double h) {
        for (int i = 0; i < nd; i++) p.r[i] += h * p.vhat[i];
    }
    void drift_r_and_kick(Part &p, double h) {
        for (int i = 0; i < nd; i++) p.r[i] += h * p.vhat[i];
        if (p.iam != T_SPHB) {
            for (int i = 0; i < nd; i++) {
                p.v0[i] = p.v[i];
                p.vhat0[i] = p.vhat[i];
                p.v[i] += h * p.f[i];
                p.vhat[i] += h * p.f[i];
            }
        }
    }
    void drift_rest(Part &p, double h) {
        p.dens += h * p.dddt;
        if (!(c.flags & SPHDEM_F_CONST_H)) p.h = c.hfac * std::pow(p.mass / p.dens, 1.0 / nd);
    }
    void kick(Part &p, double h0, double h1) {
        const double d = h0 + h1;
        if (p.iam == T_SPH || p.iam == T_DEM || p.iam == 13) {
            for (int i = 0; i < nd; i++) {
                p.v[i] = p.v0[i] + d * p.f[i];
                p.vhat[i] = p.vhat0[i] + d * p.f[i];
            }
            if (time < c.damptime)
                for (int i = 0; i < nd; i++) {
                    p.v[i] *= 0.98;
                    p.vhat[i] *= 0.98;
                }
        }
    }
    void init_sums_middle(Part &p) {
        for (int i = 0; i < 3; i++) p.f[i] = p.fp[i] = p.fv[i] = p.fb[i] = p.ff[i] = 0.0;
    }

    /* ---------------- pair physics ---------------- */
    void calc_press(Part &p) {
        if (liq_dem())
            p.press = c.prb * (std::pow(p.dens / (c.refd * p.porosity), c.gamma) - 1.0);
        else
            p.press = c.prb * (std::pow(p.dens / c.refd, 7) - 1.0);
        p.pdr2 = p.press / (p.dens * p.dens);
    }

    void calc_omega(Part &p, const std::vector<Entry> &nb) {
        p.omega = p.mass * pdWh(0, p.h);
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            if (pn.iam == T_SPH || pn.iam == T_SPHB) {
                double rb[3], dr[3];
                epos(e, rb);
                for (int i = 0; i < nd; i++) dr[i] = p.r[i] - rb[i];
                const double r = len(dr);
                p.omega += pn.mass * pdWh(r / p.h, p.h);
            }
        }
        p.omega = 1 + p.h * p.omega / (p.dens * nd);
    }

    /* inverseSym, vect.h:49-111: adjugate over determinant, identity if singular */
    void inverse_sym(double *a) const {
        if (nd == 2) {
            const double A = a[0], B = a[1], C = a[2], D = a[3];
            const double det = (A * D - B * C);
            if (det != 0.0) {
                a[0] = D / det;
                a[1] = -B / det;
                a[2] = -C / det;
                a[3] = A / det;
            } else {
                a[0] = 1.0; a[1] = 0.0; a[2] = 0.0; a[3] = 1.0;
            }
            return;
        }
        if (nd == 1) {   /* not defined by the reference (2D and 3D only) */
            a[0] = a[0] != 0.0 ? 1.0 / a[0] : 1.0;
            return;
        }
        const double A0 = a[0], B0 = a[1], C0 = a[2], D0 = a[3], E0 = a[4], F0 = a[5], G0 = a[6], H0 = a[7],
                     K0 = a[8];
        const double cA = (E0 * K0 - F0 * H0), cB = (F0 * G0 - D0 * K0), cC = (D0 * H0 - E0 * G0);
        const double cD = (C0 * H0 - B0 * K0), cE = (A0 * K0 - C0 * G0), cF = (B0 * G0 - A0 * H0);
        const double cG = (B0 * F0 - C0 * E0), cH = (C0 * D0 - A0 * F0), cK = (A0 * E0 - B0 * D0);
        const double Z = A0 * (E0 * K0 - F0 * H0) + B0 * (F0 * G0 - K0 * D0) + C0 * (D0 * H0 - E0 * G0);
        if (Z != 0) {
            const double o[9] = {cA, cD, cG, cB, cE, cH, cC, cF, cK};
            for (int k = 0; k < 9; k++) a[k] = o[k] / Z;
        } else {
            for (int k = 0; k < 9; k++) a[k] = (k % 4 == 0) ? 1.0 : 0.0;
        }
    }

    /* calcInvM, sph.h:393-434 */
    void calc_invm(Part &p, const std::vector<Entry> &nb) {
        for (int k = 0; k < 9; k++) p.invM[k] = 0.0;
        p.sum = (p.mass / p.dens) * Wk(0, p.h);
        for (int i = 0; i < 3; i++) p.sumGrad[i] = 0.0;
        if (nb.empty()) {
            for (int i = 0; i < nd; i++) p.invM[nd * i + i] = 1.0;
            return;
        }
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            if (!sph_or_sphb(pn.iam)) continue;
            double rb[3], dr[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dr[i] = p.r[i] - rb[i];
            const double r = len(dr);
            const double dvol = pn.mass / pn.dens;
            const double hav = 0.5 * (p.h + pn.h);
            const double q = r / hav;
            const double Fa = F(q, hav);
            const double Wab = Wk(q, hav);
            p.sum += dvol * Wab;
            for (int i = 0; i < nd; i++) p.sumGrad[i] += (dvol * dr[i]) * Fa;
        }
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            if (!sph_or_sphb(pn.iam)) continue;
            double rb[3], dr[3] = {0, 0, 0}, g[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dr[i] = p.r[i] - rb[i];
            const double r = len(dr);
            const double dvol = pn.mass / pn.dens;
            const double hav = 0.5 * (p.h + pn.h);
            const double Fa = F(r / hav, hav);
            for (int i = 0; i < nd; i++) g[i] = (dr[i] * Fa - p.sumGrad[i] / p.sum) / p.sum;
            for (int i = 0; i < nd; i++)
                for (int j = 0; j < nd; j++) p.invM[i * nd + j] -= (pn.mass / pn.dens) * (g[i] * dr[j]);
        }
        inverse_sym(p.invM);
    }

    /* the density re-initialisation of start(), sphIncompress.cpp:19-35:
     * a reset, then ten rounds of calcHFromDens (sph.h:1823-1825) and
     * calcDensity (sph.h:1172-1184).  The neighbour lists are built on their
     * first use, after the first calcHFromDens (dataLL.impl.h:230-240). */
    void reinit_density() {
        reset();
        const int n = ps.size();
        for (int it = 0; it < 10; it++) {
            for (auto &p : ps)
                if (p.alive && sph_or_sphb(p.iam)) p.h = c.hfac * std::pow(p.mass / p.dens, 1.0 / nd);
            if (it == 0) {
                nbrs.assign(n, std::vector<Entry>());
                for (int k : order) calc_neighbours(k, nbrs[k]);
            }
            for (int k = 0; k < n; k++) {
                Part &p = ps[k];
                if (!p.alive || !sph_or_sphb(p.iam)) continue;
                p.dens = p.mass * Wk(0, p.h);
                for (const Entry &e : nbrs[k]) {
                    const Part &pn = ps[e.idx];
                    if (!sph_or_sphb(pn.iam)) continue;
                    double rb[3], dr[3] = {0, 0, 0};
                    epos(e, rb);
                    for (int i = 0; i < nd; i++) dr[i] = p.r[i] - rb[i];
                    const double r = len(dr);
                    p.dens += pn.mass * Wk(r / p.h, p.h);
                }
            }
        }
    }
    bool reinit_due() const {
        return (c.reinit_dens_every > 0 && step % c.reinit_dens_every == 0) ||
               (c.reinit_dens_at > 0 && step == c.reinit_dens_at);
    }

    void visc_force(Part &pa, const Part &pb, const double *dx, const double *gw, const double *dv, double r) {
        const double vdr = dot(dx, dv, nd);
        const double hav = 0.5 * (pa.h + pb.h);
        double fv[3] = {0, 0, 0};
        double vsig = 0.0;
        if (c.visc_model == SPHDEM_VISC_MORRIS) {
            double visc = c.viscosity * (pa.dens + pb.dens) / (pa.dens * pb.dens);
            vsig = 2.0 * c.spsound;
            if (liq_dem()) visc = 2.0 * c.viscosity * c.dens / (pa.dens * pb.dens);
            const double dg = dot(dx, gw, nd);
            const double den = std::pow(r, 2) + 0.01 * std::pow(hav, 2);
            for (int i = 0; i < nd; i++) fv[i] = dv[i] * pb.mass * visc * dg / den;
        } else if (c.visc_model == SPHDEM_VISC_MONAGHAN) {
            double dr = 0.0;
            if (r != 0.0) dr = 1 / r;
            const double viss = vdr * dr;
            if (!liq_dem()) vsig = 2.0 * c.spsound + 2.0 * std::fabs(viss);
            const double alpha = c.viscosity * (112.0 / 15.0) / (c.spsound * c.h);
            const double visc = viss * vsig * alpha / (pa.dens + pb.dens);
            for (int i = 0; i < nd; i++) fv[i] = pb.mass * visc * gw[i];
        } else if (c.visc_model == SPHDEM_VISC_ARTIFICIAL) {
            double avsig = 0, avisc = 0.0;
            if (vdr < 0) {
                double dr = 0.0;
                if (r != 0.0) dr = 1 / r;
                const double viss = vdr * dr;
                avsig = 2.0 * c.spsound - 4.0 * viss;
                avisc = viss * avsig * c.alpha_artificial / (pa.dens + pb.dens);
            }
            for (int i = 0; i < nd; i++) pa.f[i] += pb.mass * avisc * gw[i];
            vsig = std::max(vsig, avsig);
        }
        newDt = std::min(newDt, 0.6 * hav / vsig);
        const double vdc = c.visc_model == SPHDEM_VISC_MONAGHAN ? 0.06 : 0.125;
        newDt = std::min(newDt, vdc * std::pow(hav, 2) / c.viscosity);
        for (int i = 0; i < nd; i++) {
            pa.fv[i] += fv[i];
            pa.f[i] += fv[i];
        }
    }

    void calc_normal(const Part &pb, const double *dx, double r, double *normp, double *normt) {
        const bool n2zero = pb.norm2[0] == 0 && pb.norm2[1] == 0 && (nd < 3 || pb.norm2[2] == 0);
        for (int i = 0; i < 3; i++) normt[i] = pb.norm3[i];
        if (n2zero) {
            for (int i = 0; i < 3; i++) normp[i] = pb.norm1[i];
            return;
        }
        const float rdot1 = dot(dx, pb.norm1, nd);
        const float rdot2 = dot(dx, pb.norm2, nd);
        const float rntest = r * r * dot(pb.norm1, pb.norm2, nd) - rdot1 * rdot2;
        if (rntest <= 0) {
            for (int i = 0; i < nd; i++) normp[i] = dx[i] / r;
            return;
        }
        const int con = pb.concave ? 1 : -1;
        if (con * (rdot1 - rdot2) > 0)
            for (int i = 0; i < 3; i++) normp[i] = pb.norm1[i];
        else
            for (int i = 0; i < 3; i++) normp[i] = pb.norm2[i];
    }

    /* calcBoundaryForces, sph.h:789-918 (MODIFY_BFORCE_WITH_STILL_LEVEL off) */
    void boundary_force(Part &p, const Part &bp, const double *rb, const double *normp, const double *normt) {
        double dx[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
        for (int i = 0; i < nd; i++) {
            dx[i] = p.r[i] - rb[i];
            dv[i] = p.vhat[i] - bp.vhat[i];
        }
        const double rperp = dot(normp, dx, nd);
        double rtang[3] = {0, 0, 0};
        for (int i = 0; i < nd; i++) rtang[i] = dx[i] - rperp * normp[i];
        double pt0, pt1;
        const double rDelP = 1.0 / (c.bfac * c.psep);
        if (nd == 3) {
            pt0 = std::fabs(dot(rtang, normt, 3));
            double cr[3] = {rtang[1] * normt[2] - rtang[2] * normt[1],
                            rtang[2] * normt[0] - rtang[0] * normt[2],
                            rtang[0] * normt[1] - rtang[1] * normt[0]};
            pt1 = len(cr);
        } else {
            pt0 = len(rtang);
            pt1 = 0;
        }
        const double pd0 = pt0 * rDelP, pd1 = pt1 * rDelP;
        if (pd0 <= 1.0 && pd1 <= 1.0) {
            const double pesky = 0.25 * (1 + std::cos(c.pi * pd0)) * (1 + std::cos(c.pi * pd1));
            const double q = std::fabs(rperp) / (1.0 * c.psep);
            double fb[3] = {0, 0, 0};
            if (q < 2.0) {
                const double epsilon = 1;
                int beta = 0;
                if (dot(dx, dv, nd) < 0) beta = 1;
                const double bigA = 0.01 * std::pow(c.spsound, 2) - beta * c.spsound * dot(dv, normp, nd);
                const double bfact = 1.0 / std::fabs(rperp);
                const double QIN = 2.0 / 3.0;
                double bforce = 0.0;
                if (q <= QIN) bforce = bfact * QIN;
                else if (q <= 1.0) bforce = bfact * (2.0 * q - 1.5 * q * q);
                else if (q <= 2.0) bforce = bfact * 0.5 * std::pow(2.0 - q, 2);
                const double bigR = bigA * bforce;
                const double amassrat = 2.0 * p.mass / (p.mass + bp.mass);
                int sign = 1;
                if (rperp < 0) sign = -1;
                for (int i = 0; i < nd; i++) fb[i] = sign * amassrat * normp[i] * bigR * pesky * epsilon;
            }
            for (int i = 0; i < nd; i++) {
                p.fb[i] += fb[i];
                p.f[i] += fb[i];
            }
        }
    }

    /* calcForce, sphIncompress.h:899-972 */
    void calc_force(Part &pa, const Entry &e) {
        const Part &pb = ps[e.idx];
        double rb[3], dx[3] = {0, 0, 0};
        epos(e, rb);
        for (int i = 0; i < nd; i++) dx[i] = pa.r[i] - rb[i];
        const double r = len(dx);
        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gwa[3] = {0, 0, 0}, gwb[3] = {0, 0, 0};
        gradW(pa, dx, r / pa.h, pa.h, gA);
        gradW(pa, dx, r / pb.h, pb.h, gB);
        if (var_h()) {
            for (int i = 0; i < nd; i++) { gwa[i] = gA[i]; gwb[i] = gB[i]; }
        } else {
            for (int i = 0; i < nd; i++) gwa[i] = gwb[i] = 0.5 * (gA[i] + gB[i]);
        }
        if (pa.iam == T_SPH && pb.iam != T_DEM && pb.iam != 12) {
            double dv[3] = {0, 0, 0}, gm[3] = {0, 0, 0};
            for (int i = 0; i < nd; i++) {
                dv[i] = pa.vhat[i] - pb.vhat[i];
                gm[i] = 0.5 * (gwa[i] + gwb[i]);
            }
            visc_force(pa, pb, dx, gm, dv, r);
        }
        double kdwPowNeps = 0.0;
        if (!(c.flags & SPHDEM_F_NO_ANTICLUMPING)) {
            const double hav = 0.5 * (pa.h + pb.h);
            const double q = r / hav;
            const double kdw = K(q) / K(1.0 / c.hfac);
            kdwPowNeps = std::pow(kdw, 4);
        }
        if (is_boundary(pb.iam)) {
            double normp[3] = {0, 0, 0}, normt[3] = {0, 0, 0};
            calc_normal(pb, dx, r, normp, normt);
            boundary_force(pa, pb, rb, normp, normt);
        } else if (pb.iam == T_SPH || pb.iam == T_SPHB) {
            const double antic = 0.01 * std::fabs(pa.pdr2 + pb.pdr2) * kdwPowNeps;
            for (int i = 0; i < nd; i++) {
                double prfac = pa.pdr2 * gwa[i] + pb.pdr2 * gwb[i];
                prfac = prfac + antic;
                const double fp = -pb.mass * prfac;
                pa.fp[i] += fp;
                pa.f[i] += fp;
            }
        }
    }

    /* calcDddtDudt, sphIncompress.h:783-851 */
    void calc_dddt(Part &pa, const Entry &e) {
        const Part &pb = ps[e.idx];
        if (is_boundary(pb.iam) || pb.iam == T_DEM) return;
        double rb[3], dr[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
        epos(e, rb);
        for (int i = 0; i < nd; i++) {
            dr[i] = pa.r[i] - rb[i];
            dv[i] = pa.vhat[i] - pb.vhat[i];
        }
        const double r = len(dr);
        double g[3] = {0, 0, 0};
        if (var_h()) {
            gradW(pa, dr, r / pa.h, pa.h, g);
        } else {
            double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
            gradW(pa, dr, r / pa.h, pa.h, gA);
            gradW(pa, dr, r / pb.h, pb.h, gB);
            for (int i = 0; i < nd; i++) g[i] = 0.5 * (gA[i] + gB[i]);
        }
        const double vdr = dot(dv, g, nd);
        pa.dddt += pb.mass * vdr;
    }

    /* ---------------- coupling, sph.h:1246-1362, 1575-1792 ---------------- */
    double porosity_incr(double w) const {
        if (nd == 2) return (4.0 / 3.0) * c.pi * std::pow(c.dem_radius, 3) * w / (2.0 * c.dem_radius);
        return (4.0 / 3.0) * c.pi * std::pow(c.dem_radius, 3) * w;
    }

    void calc_porosity(Part &p, const std::vector<Entry> &nb) {
        p.porosity = 0;
        p.dpordt = 0;
        for (int i = 0; i < 3; i++) p.gradPor[i] = 0;
        const double hc = c.coupling_radius / 2.0;
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            double rb[3], dx[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dx[i] = p.r[i] - rb[i];
            const double r = len(dx);
            const double q = r * (2.0 / c.coupling_radius);
            const double Wa = Wk(q, hc);
            p.porosity += porosity_incr(Wa);
            if (r != 0.0) {
                double dv[3] = {0, 0, 0};
                for (int i = 0; i < nd; i++) dv[i] = p.vhat[i] - pn.vhat[i];
                const double fq = F(q, hc);
                p.dpordt -= c.dem_vol * dot(dv, dx, nd) * fq;
                for (int i = 0; i < nd; i++) p.gradPor[i] += c.dem_vol * dx[i] * fq;
            }
        }
    }

    void calc_shep_scatter(const Part &p, const std::vector<Entry> &nb) {
        const double dvol = p.mass / p.dens;
        for (const Entry &e : nb) {
            Part &pn = ps[e.idx];
            double rb[3], dx[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dx[i] = p.r[i] - rb[i];
            const double r = len(dx);
            pn.shep += dvol * Wk(r * (2.0 / c.coupling_radius), c.coupling_radius / 2.0);
        }
    }

    void calc_dem_to_sph_drag(Part &p, const std::vector<Entry> &nb) {
        for (int i = 0; i < 3; i++) p.fdrag[i] = 0.0;
        const double rdens = nd == 2 ? (1.0 / (2.0 * c.dem_radius)) / p.dens : 1.0 / p.dens;
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            double rb[3], dx[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dx[i] = p.r[i] - rb[i];
            const double r = len(dx);
            const double w = Wk(r * (2.0 / c.coupling_radius), c.coupling_radius / 2.0);
            for (int i = 0; i < nd; i++) p.fdrag[i] -= pn.mass * rdens * pn.fdrag[i] * w / pn.shep;
        }
        for (int i = 0; i < nd; i++) p.f[i] += p.fdrag[i];
    }

    void particle_drag(const Part &p, const double *fvel, double *out) {
        double dv[3] = {0, 0, 0};
        for (int i = 0; i < nd; i++) dv[i] = p.porosity * (fvel[i] - p.vhat[i]);
        const double vdiff = len(dv);
        double fd[3] = {0, 0, 0};
        if (vdiff != 0) {
            const double A = c.pi * std::pow(c.dem_radius, 2);
            const double Re = (2.0 * c.dem_radius / c.viscosity) * vdiff;
            const double dragGamma = 3.7 - 0.65 * std::exp(-std::pow(1.5 - std::log10(Re), 2) / 2.0);
            const double C = std::pow(0.63 + 4.8 / std::pow(Re, 0.5), 2);
            const double s = (1.0 / 2.0) * A * C * vdiff;
            const double pw = std::pow(p.porosity, -dragGamma);
            for (int i = 0; i < nd; i++) fd[i] = s * dv[i] * pw;
        }
        for (int i = 0; i < nd; i++) out[i] = (c.dens / p.mass) * fd[i];
    }

    void calc_fpi(Part &p, const std::vector<Entry> &nb) {
        double sum = 0, fdens = 0;
        double ff[3] = {0, 0, 0}, fpfb[3] = {0, 0, 0}, fv[3] = {0, 0, 0}, fdrag[3] = {0, 0, 0};
        for (int i = 0; i < 3; i++) p.fvel[i] = p.fdrag[i] = 0.0;
        p.porosity = 0.0;
        p.shep = 0.0;
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            if (pn.iam == T_BOUNDARY) continue;
            double rb[3], dx[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) dx[i] = p.r[i] - rb[i];
            const double r = len(dx);
            const double dvol = pn.mass / pn.dens;
            const double q = r / pn.h;
            const double Wab = Wk(q, pn.h);
            const double dvWab = dvol * Wab;
            for (int i = 0; i < nd; i++) {
                fpfb[i] += pn.mass * Wab * (pn.fp[i] + pn.fb[i]);
                fv[i] += pn.mass * Wab * (pn.fv[i]);
                fv[i] += dvWab * (pn.fv[i]);
                ff[i] += dvWab * (pn.f[i]);
                fdrag[i] += dvWab * pn.fdrag[i];
                p.fvel[i] += dvWab * pn.vhat[i];
            }
            p.porosity += dvWab * pn.porosity;
            fdens += Wab * pn.mass;
            sum += dvWab;
        }
        p.shep = sum;
        if (p.shep > 0.5) {
            const double rsum = 1.0 / sum;
            for (int i = 0; i < nd; i++) {
                ff[i] *= rsum;
                fpfb[i] *= rsum;
                fv[i] *= rsum;
                fdrag[i] *= rsum;
                p.fvel[i] *= rsum;
            }
            fdens *= rsum;
            p.porosity *= rsum;
            for (int i = 0; i < nd; i++) {
                p.fb[i] = fpfb[i];
                p.fv[i] = fv[i];
            }
            double dvF[3] = {0, 0, 0};
            particle_drag(p, p.fvel, dvF);
            for (int i = 0; i < nd; i++) {
                p.fdrag[i] = (c.dem_vol / p.mass) * (fv[i] + fpfb[i]) + dvF[i];
                p.f[i] += p.fdrag[i];
            }
        }
    }

    double radius_of(const Part &p) const { return p.radius > 0 ? p.radius : c.dem_radius; }

    /* calcDEMContacts, sph.h:1676-1706 (LINEAR demNormal, sph.h:1513-1515) */
    void calc_dem_contacts(Part &p, const std::vector<Entry> &nb) {
        for (const Entry &e : nb) {
            const Part &pn = ps[e.idx];
            double rb[3], dx[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, nrm[3] = {0, 0, 0};
            epos(e, rb);
            for (int i = 0; i < nd; i++) {
                dx[i] = p.r[i] - rb[i];
                dv[i] = p.vhat[i] - pn.vhat[i];
            }
            const double r = len(dx);
            for (int i = 0; i < nd; i++) nrm[i] = dx[i] / r;
            const double overlap = (radius_of(p) + radius_of(pn)) - r;
            if (overlap > 0) {
                const double od = -dot(dv, nrm, nd);
                const double s = c.dem_k * overlap + c.dem_gamma * od;
                for (int i = 0; i < nd; i++) {
                    const double fN = (s * nrm[i]) / p.mass;
                    p.fp[i] += fN;
                    p.f[i] += fN;
                }
            }
        }
    }

    /* ---------------- built-in hooks (customSim pattern) ---------------- */
    void hook_before_middle() {
        for (auto &p : ps)
            if (p.alive && p.iam == T_SPH)
                for (int i = 0; i < nd; i++)
                    if (c.gravity_sph[i] != 0.0) p.f[i] += c.gravity_sph[i];
    }
    void hook_before_end() {
        if (!liq_dem()) return;
        for (auto &p : ps) {
            if (!p.alive || p.iam != T_DEM) continue;
            for (int i = 0; i < nd; i++)
                if (c.gravity_dem[i] != 0.0) p.f[i] += c.gravity_dem[i];
        }
        for (auto &p : ps) {
            if (!p.alive || p.iam != T_DEM) continue;
            for (int w = 0; w < c.n_walls; w++) {
                const SphDemWall &wl = c.walls[w];
                double d[3] = {0, 0, 0};
                for (int i = 0; i < nd; i++) d[i] = p.r[i] - wl.point[i];
                const double overlap = radius_of(p) - dot(d, wl.normal, nd);
                if (overlap > 0.0) {
                    const double od = -dot(p.vhat, wl.normal, nd);
                    const double s = c.dem_k * overlap + c.dem_gamma * od;
                    for (int i = 0; i < nd; i++) {
                        const double fN = (s * wl.normal[i]) / p.mass;
                        p.fb[i] += fN;
                        p.f[i] += fN;
                    }
                }
            }
        }
        freeze();
    }
    void freeze() {
        if (!liq_dem() || !(time <= c.freeze_dem_until)) return;
        for (auto &p : ps)
            if (p.alive && p.iam == T_DEM)
                for (int i = 0; i < 3; i++) p.f[i] = p.v[i] = p.vhat[i] = 0.0;
    }

    /* ---------------- phases, sphIncompress.cpp:3-251 ---------------- */
    void start() {
        const double h = dt / 2;
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) drift_r_and_kick(p, h);
        if (liq_dem())
            for (auto &p : ps)
                if (p.alive && p.iam == T_DEM) drift_r(p, h);
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) drift_rest(p, h);
        time += dt / 2;
        if (reinit_due()) reinit_density();
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) init_sums_middle(p);
    }

    void middle() {
        newDt = maxdt;
        reset();
        const int n = ps.size();
        if (liq_dem()) {
            std::vector<std::vector<Entry>> cn(n);
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) {
                    calc_coupling(k, cn[k]);
                    calc_porosity(ps[k], cn[k]);
                }
            for (auto &p : ps)
                if (p.iam == T_DEM) p.shep = 0.0;
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_shep_scatter(ps[k], cn[k]);
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_dem_to_sph_drag(ps[k], cn[k]);
            for (auto &p : ps) {
                if (!p.alive) continue;
                if (sph_or_sphb(p.iam)) {
                    p.porosity = 1.0 - p.porosity;
                    if (p.porosity < 0.37) {
                        p.porosity = 0.37;
                        p.dpordt = 0.0;
                        for (int i = 0; i < 3; i++) p.gradPor[i] = 0.0;
                    }
                }
            }
            for (auto &p : ps)
                if (p.alive && is_boundary(p.iam)) p.porosity = 1.0;
        }
        if (corrected())
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_invm(ps[k], nbrs[k]);
        if (var_h())
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_omega(ps[k], nbrs[k]);
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) calc_press(p);
        for (int k = 0; k < n; k++)
            if (ps[k].alive && sph_or_sphb(ps[k].iam))
                for (const Entry &e : nbrs[k]) calc_force(ps[k], e);
        if (liq_dem()) {
            newDt = std::min(newDt, c.liq_dem_timestep);
            if (time > c.time_drop_particle) newDt = std::min(newDt, c.dem_timestep);
        }
        for (auto &p : ps)
            if (p.alive && (sph_or_sphb(p.iam) || p.iam == T_DEM))
                newDt = std::min(newDt, 0.25 * std::sqrt(p.h / len(p.f)));
        const double oldDt = dt;
        if (c.flags & SPHDEM_F_FIXED_DT) dt = maxdt;
        else dt = newDt;
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) kick(p, 0.5 * oldDt, 0.5 * dt);
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) p.dddt = 0.0;
        if (liq_dem()) {
            for (auto &p : ps)
                if (p.alive && p.iam == T_DEM) drift_r_and_kick(p, dt / 2);
            for (auto &p : ps)
                if (p.alive && p.iam == T_DEM) init_sums_middle(p);
        }
    }

    void end() {
        if (liq_dem()) demDt = maxdt;
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) drift_r(p, dt / 2);
        time += dt / 2;
        reset();
        const int n = ps.size();
        if (corrected())
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_invm(ps[k], nbrs[k]);
        if (var_h())
            for (int k = 0; k < n; k++)
                if (ps[k].alive && sph_or_sphb(ps[k].iam)) calc_omega(ps[k], nbrs[k]);
        for (int k = 0; k < n; k++)
            if (ps[k].alive && sph_or_sphb(ps[k].iam))
                for (const Entry &e : nbrs[k]) calc_dddt(ps[k], e);
        if (liq_dem()) {
            std::vector<Entry> cn;
            for (int k = 0; k < n; k++)
                if (ps[k].alive && ps[k].iam == T_DEM) {
                    cn.clear();
                    calc_coupling(k, cn);
                    calc_fpi(ps[k], cn);
                }
            for (int k = 0; k < n; k++)
                if (ps[k].alive && ps[k].iam == T_DEM) calc_dem_contacts(ps[k], nbrs[k]);
            if (c.flags & SPHDEM_F_DEM_BLOCK) {
                /* DEM_BLOCK, sphIncompress.cpp:231-238: calcAvForce, mean, setAvForce
                 * (sphIncompress.h:107-114), in traverse order */
                double av[3] = {0, 0, 0}, cnt = 0;
                for (int k : order)
                    if (ps[k].alive && ps[k].iam == T_DEM) {
                        for (int i = 0; i < 3; i++) av[i] += ps[k].f[i];
                        cnt++;
                    }
                for (int i = 0; i < 3; i++) av[i] = av[i] / cnt;
                for (auto &p : ps)
                    if (p.alive && p.iam == T_DEM)
                        for (int i = 0; i < 3; i++) p.f[i] = av[i];
            }
            for (auto &p : ps)
                if (p.alive && p.iam == T_DEM) kick(p, 0.5 * dt, 0.5 * dt);
        }
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) drift_rest(p, dt / 2);
        /* calcEnergies (sphIncompress.h:769-781): press/pdr2 refresh, elastic
         * energy, and the viscous energy of sph particles */
        for (auto &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) {
                if (p.iam == T_SPH) {
                    p.deViscFdt = -dot(p.vhat, p.fv, nd);
                    p.eViscF += dt * p.deViscFdt;
                }
                calc_press(p);
                p.dudt = p.pdr2 * p.dddt;
                p.u += dt * p.dudt;
            }
    }

    /* calcOutputVars (sphIncompress.h:274-319): calcOutput over sph /
     * sphBoundary (233-262), calcAveDensFromMass over the cached neighbour
     * lists (266-272 with calcDensity, sph.h:1149-1191), calcVarDens (264) */
    void output_vars(SphDemOutputVars &o) const {
        o = SphDemOutputVars{};
        double aveDens = 0, dfm = 0;
        long long nlive = 0, nsph = 0;
        for (size_t k = 0; k < ps.size(); k++) {
            const Part &p = ps[k];
            if (!p.alive) continue;
            nlive++;
            if (!sph_or_sphb(p.iam)) continue;
            if (p.iam == T_SPH) {
                for (int i = 0; i < nd; i++) o.lin_mom[i] += p.v[i] * p.mass;
                o.ang_mom += (p.r[0] * p.v[1] - p.r[1] * p.v[0]) * p.mass;
                o.e_ke += 0.5 * p.mass * len2(p.vhat);
                o.e_visc_f += p.mass * p.eViscF;
                o.ed_visc_f_dt += p.mass * p.deViscFdt;
                nsph++;
            }
            o.max_v = std::max(o.max_v, len(p.v));
            o.max_f = std::max(o.max_f, len(p.f));
            aveDens += p.dens;
            o.e_elast += p.mass * p.u;
            o.ed_elast_dt += p.mass * p.dudt;
            const double x = p.dens / c.refd;
            o.e_elast_exact += p.mass * (c.prb * ((std::pow(x, 6) - 1) / 6 + 1 / x - 1)) / c.refd;
            double rho = p.mass * Wk(0.0, p.h);
            for (const Entry &e : nbrs[k]) {
                const Part &pb = ps[e.idx];
                if (!sph_or_sphb(pb.iam)) continue;
                double rb[3], dr[3] = {0, 0, 0};
                epos(e, rb);
                for (int i = 0; i < nd; i++) dr[i] = p.r[i] - rb[i];
                rho += pb.mass * Wk(len(dr) / p.h, p.h);
            }
            dfm += (rho - p.dens) * (rho - p.dens);
        }
        o.n = nlive;
        o.n_sph = nsph;
        o.ave_dens = aveDens / nlive;
        o.ave_dens_from_mass = std::sqrt(dfm / nlive);
        double var = 0;
        for (const Part &p : ps)
            if (p.alive && sph_or_sphb(p.iam)) var += (p.dens - o.ave_dens) * (p.dens - o.ave_dens);
        o.var_dens = var / nlive;
        o.e_total = o.e_ke + o.e_elast + o.e_visc_f + o.e_visc_b + o.e_b_force + o.e_ff;
    }

    void full_step() {
        step++;
        start();
        hook_before_middle();
        middle();
        hook_before_end();
        end();
        freeze();
    }
};

std::string g_err;

/* a particle as the Cparticle constructor and the case set it (particle.h:60-120) */
void init_part(Part &p, const SphDemParticles *in, int64_t k) {
    std::memset(&p, 0, sizeof(Part));
    p.alive = true;
    p.iam = in->iam[k];
    p.tag = in->tag ? in->tag[k] : (int)k + 1;
    p.concave = in->concave ? in->concave[k] != 0 : true;
    for (int i = 0; i < 3; i++) {
        p.r[i] = in->r[3 * k + i];
        p.v[i] = in->v ? in->v[3 * k + i] : 0.0;
        p.vhat[i] = in->vhat ? in->vhat[3 * k + i] : p.v[i];
        p.norm1[i] = in->norm1 ? in->norm1[3 * k + i] : 0.0;
        p.norm2[i] = in->norm2 ? in->norm2[3 * k + i] : 0.0;
        p.norm3[i] = in->norm3 ? in->norm3[3 * k + i] : 0.0;
    }
    p.mass = in->mass[k];
    p.dens = in->dens[k];
    p.h = in->h[k];
    p.radius = in->radius ? in->radius[k] : 0.0;
    p.porosity = 1.0;
}

void load(Sim &s, const SphDemConfig *cfg, const SphDemParticles *in) {
    s.c = *cfg;
    s.nd = cfg->ndim;
    s.wcon = s.nd == 2 ? 7.0 / (64.0 * cfg->pi) : 21.0 / (256.0 * cfg->pi);
    s.maxdt = cfg->maxdt;
    s.dt = cfg->maxdt;
    s.ps.resize(in->n);
    for (int64_t k = 0; k < in->n; k++) init_part(s.ps[k], in, k);
    s.init_grids();
    s.reset();
}

}  // namespace

extern "C" {

int oracle_create(const SphDemConfig *cfg, const SphDemParticles *init, void **out) {
    try {
        Sim *s = new Sim();
        load(*s, cfg, init);
        *out = s;
        return 0;
    } catch (const std::string &e) {
        g_err = e;
        return SPHDEM_ERR_INVALID;
    }
}

void oracle_destroy(void *h) { delete static_cast<Sim *>(h); }

int oracle_step(void *h, int nsteps) {
    Sim *s = static_cast<Sim *>(h);
    try {
        for (int k = 0; k < nsteps; k++) s->full_step();
    } catch (const std::string &e) {
        g_err = e;
        return SPHDEM_ERR_OUT_OF_RANGE;
    }
    return 0;
}

/* Run one phase / hook point, numbered as SPHDEM_PHASE_* / SPHDEM_HOOK_*. */
int oracle_phase(void *h, int phase) {
    Sim *s = static_cast<Sim *>(h);
    try {
        switch (phase) {
            case SPHDEM_HOOK_BEFORE_START: s->step++; break;
            case SPHDEM_PHASE_START: s->start(); break;
            case SPHDEM_HOOK_BEFORE_MIDDLE: s->hook_before_middle(); break;
            case SPHDEM_PHASE_MIDDLE: s->middle(); break;
            case SPHDEM_HOOK_BEFORE_END: s->hook_before_end(); break;
            case SPHDEM_PHASE_END: s->end(); break;
            case SPHDEM_HOOK_AFTER_END: s->freeze(); break;
            default: return SPHDEM_ERR_INVALID;
        }
    } catch (const std::string &e) {
        g_err = e;
        return SPHDEM_ERR_OUT_OF_RANGE;
    }
    return 0;
}

/* CdataLL::reset at the current positions (the pair exports read the
 * buckets of the last reset). */
/* insertNewParticle (dataLL.cpp:238-261): appended to the container
 * (traversal) order; the index is the lowest dead slot, else the next */
int oracle_insert(void *h, const SphDemParticles *in, int64_t *out_idx) {
    Sim *s = static_cast<Sim *>(h);
    size_t cursor = 0;
    for (int64_t j = 0; j < in->n; j++) {
        while (cursor < s->ps.size() && s->ps[cursor].alive) cursor++;
        const size_t slot = cursor < s->ps.size() ? cursor++ : s->ps.size();
        if (slot == s->ps.size()) s->ps.emplace_back();
        init_part(s->ps[slot], in, j);
        s->order.push_back((int)slot);
        if (out_idx) out_idx[j] = (int64_t)slot;
    }
    return 0;
}

/* markForDeletion (dataLL.cpp:263-266) */
int oracle_mark_for_deletion(void *h, const int64_t *idx, int64_t k) {
    Sim *s = static_cast<Sim *>(h);
    for (int64_t j = 0; j < k; j++) {
        if (idx[j] < 0 || idx[j] >= (int64_t)s->ps.size() || !s->ps[idx[j]].alive) {
            g_err = "bad deletion index";
            return 1;
        }
    }
    for (int64_t j = 0; j < k; j++) s->ps[idx[j]].marked = true;
    return 0;
}

int oracle_rebuild(void *h) {
    Sim *s = static_cast<Sim *>(h);
    try {
        s->reset();
    } catch (const std::string &e) {
        g_err = e;
        return SPHDEM_ERR_OUT_OF_RANGE;
    }
    return 0;
}

int oracle_get(void *h, SphDemParticles *o) {
    Sim *s = static_cast<Sim *>(h);
    const int n = s->ps.size();
    if (o->n != n) return SPHDEM_ERR_INVALID;
    for (int k = 0; k < n; k++) {
        const Part &p = s->ps[k];
        auto put3 = [&](double *dst, const double *src) {
            if (dst) for (int i = 0; i < 3; i++) dst[3 * k + i] = src[i];
        };
        auto put1 = [&](double *dst, double v) { if (dst) dst[k] = v; };
        if (o->iam) o->iam[k] = p.alive ? p.iam : -1;
        if (o->tag) o->tag[k] = p.tag;
        put3(o->r, p.r); put3(o->v, p.v); put3(o->vhat, p.vhat);
        put3(o->v0, p.v0); put3(o->vhat0, p.vhat0);
        put3(o->f, p.f); put3(o->fp, p.fp); put3(o->fv, p.fv); put3(o->fb, p.fb);
        put3(o->fdrag, p.fdrag); put3(o->fvel, p.fvel); put3(o->grad_porosity, p.gradPor);
        put1(o->mass, p.mass); put1(o->dens, p.dens); put1(o->h, p.h);
        put1(o->dddt, p.dddt); put1(o->press, p.press); put1(o->pdr2, p.pdr2);
        put1(o->porosity, p.porosity); put1(o->dporositydt, p.dpordt);
        put1(o->shep_sum, p.shep); put1(o->omega, p.omega);
        put1(o->radius, p.radius);
        put1(o->u, p.u); put1(o->dudt, p.dudt); put1(o->e_visc, p.eViscF); put1(o->de_visc_dt, p.deViscFdt);
    }
    return 0;
}

/* Write the fields the mask selects (the SPHDEM_FIELD_* groups of
 * sphdem_set_fields), container order; as a case hook writes them between
 * phases through the façade's host mirror. */
int oracle_set(void *h, uint32_t mask, const SphDemParticles *in) {
    Sim *s = static_cast<Sim *>(h);
    const int n = s->ps.size();
    if (in->n != n) return SPHDEM_ERR_INVALID;
    for (int k = 0; k < n; k++) {
        Part &p = s->ps[k];
        auto get3 = [&](double *dst, const double *src) {
            if (src) for (int i = 0; i < 3; i++) dst[i] = src[3 * k + i];
        };
        auto get1 = [&](double &dst, const double *src) { if (src) dst = src[k]; };
        if (mask & SPHDEM_FIELD_R) get3(p.r, in->r);
        if (mask & SPHDEM_FIELD_V) get3(p.v, in->v);
        if (mask & SPHDEM_FIELD_VHAT) get3(p.vhat, in->vhat);
        if (mask & SPHDEM_FIELD_MASS) get1(p.mass, in->mass);
        if (mask & SPHDEM_FIELD_DENS) get1(p.dens, in->dens);
        if (mask & SPHDEM_FIELD_H) get1(p.h, in->h);
        if (mask & SPHDEM_FIELD_F) {
            get3(p.f, in->f); get3(p.fp, in->fp); get3(p.fv, in->fv); get3(p.fb, in->fb);
        }
        if (mask & SPHDEM_FIELD_DDDT) get1(p.dddt, in->dddt);
        if (mask & SPHDEM_FIELD_PRESS) {
            get1(p.press, in->press); get1(p.pdr2, in->pdr2);
        }
        if (mask & SPHDEM_FIELD_COUPLING) {
            get1(p.porosity, in->porosity); get1(p.dpordt, in->dporositydt); get1(p.shep, in->shep_sum);
            get3(p.fdrag, in->fdrag); get3(p.fvel, in->fvel); get3(p.gradPor, in->grad_porosity);
        }
        if (mask & SPHDEM_FIELD_OMEGA) get1(p.omega, in->omega);
        if (mask & SPHDEM_FIELD_V0) {
            get3(p.v0, in->v0); get3(p.vhat0, in->vhat0);
        }
        if (mask & SPHDEM_FIELD_NORMALS) {
            get3(p.norm1, in->norm1); get3(p.norm2, in->norm2); get3(p.norm3, in->norm3);
        }
        if (mask & SPHDEM_FIELD_RADIUS) get1(p.radius, in->radius);
        if (mask & SPHDEM_FIELD_ENERGY) {
            get1(p.u, in->u); get1(p.dudt, in->dudt); get1(p.eViscF, in->e_visc); get1(p.deViscFdt, in->de_visc_dt);
        }
    }
    return 0;
}

/* time, dt, maxdt and the step count, as sphdem_set_globals sets them */
int oracle_set_globals(void *h, const SphDemGlobals *g) {
    Sim *s = static_cast<Sim *>(h);
    s->time = g->time;
    s->dt = g->dt;
    s->maxdt = g->maxdt;
    s->step = g->sph_step;
    return 0;
}

int oracle_output_vars(void *h, SphDemOutputVars *o) {
    static_cast<Sim *>(h)->output_vars(*o);
    return 0;
}

/* Neighbour relations at the current positions, CSR over container order,
 * each row sorted ascending (duplicate images collapsed). */
int oracle_pairs(void *h, int kind, int64_t *offs, int32_t *idx, int64_t cap, int64_t *npairs) {
    Sim *s = static_cast<Sim *>(h);
    const int n = s->ps.size();
    std::vector<std::vector<int>> rows(n);
    std::vector<Entry> tmp;
    const double rc2 = std::pow(s->c.coupling_radius, 2);
    for (int k = 0; k < n; k++) {
        const Part &p = s->ps[k];
        if (!p.alive) continue;
        const bool dem = s->liq_dem() && p.iam == T_DEM;
        tmp.clear();
        if (kind == SPHDEM_PAIRS_SPH && !dem) s->calc_neighbours(k, tmp);
        else if (kind == SPHDEM_PAIRS_DEM && dem) s->calc_neighbours(k, tmp);
        else if (kind == SPHDEM_PAIRS_COUPLE_DS && dem) s->calc_coupling(k, tmp);
        else if (kind == SPHDEM_PAIRS_COUPLE_SD && s->liq_dem() && Sim::sph_or_sphb(p.iam)) {
            std::vector<Entry> all;
            s->calc_coupling(k, all);
            for (const Entry &e : all) {
                double rb[3], d[3] = {0, 0, 0};
                s->epos(e, rb);
                for (int i = 0; i < s->nd; i++) d[i] = p.r[i] - rb[i];
                if (s->len2(d) < rc2) tmp.push_back(e);
            }
        }
        for (const Entry &e : tmp) rows[k].push_back(e.idx);
        std::sort(rows[k].begin(), rows[k].end());
        rows[k].erase(std::unique(rows[k].begin(), rows[k].end()), rows[k].end());
    }
    int64_t tot = 0;
    for (int k = 0; k < n; k++) {
        if (offs) offs[k] = tot;
        tot += rows[k].size();
    }
    if (offs) offs[n] = tot;
    *npairs = tot;
    if (!idx) return 0;
    if (tot > cap) return SPHDEM_ERR_CAPACITY;
    int64_t o = 0;
    for (int k = 0; k < n; k++)
        for (int v : rows[k]) idx[o++] = v;
    return 0;
}

int oracle_cells(void *h, int32_t *cells) {
    Sim *s = static_cast<Sim *>(h);
    const int n = s->ps.size();
    for (int k = 0; k < n; k++) {
        int ci[3] = {0, 0, 0};
        const Part &p = s->ps[k];
        if (s->liq_dem() && p.iam == T_DEM) s->dem_cell(p.r, ci); else s->sph_cell(p.r, ci);
        for (int i = 0; i < 3; i++) cells[3 * k + i] = ci[i];
    }
    return 0;
}

int oracle_globals(void *h, SphDemGlobals *g) {
    Sim *s = static_cast<Sim *>(h);
    g->time = s->time;
    g->dt = s->dt;
    g->new_dt = s->newDt;
    g->maxdt = s->maxdt;
    g->dem_dt = s->demDt;
    g->sph_step = s->step;
    g->n_deleted = s->n_deleted;
    return 0;
}

const char *oracle_last_error(void) { return g_err.c_str(); }

}  // extern "C"
