/*
 * CdataLL of the plug-in surface, as a host mirror of a device simulation.
 *
 * The device (include/sphdem.h) owns the particles.  The façade driver calls
 * pull() before a case hook, which copies every field of every particle
 * into `ps` (tag order: the order the particles were created in) and the
 * step globals into `globals`, and push() after it, which writes the
 * mutable fields (r, v, vhat, f/fp/fv/fb, dens, h) and the globals back.
 * traverse / neighboursGroup run the case functors on the mirror
 * (dataLL.h:125-176); neighbour lists come from the device's own list
 * (sphdem_pairs) and are fetched once per pull.  insertNewParticle and
 * markForDeletion (dataLL.cpp:238-266) queue on the mirror and reach the
 * device at push(): marked particles leave at its next rebuild, inserted
 * ones take the lowest free slots (sphdem_insert_particles), and the
 * mirror grows to the device's particle count.
 */
#ifndef DATALL_H
#define DATALL_H

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iostream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/sphdem.h"
#include "customConstants.h"
#include "globalVars.h"
#include "particle.h"
#include "vect.h"

using std::vector;

class CdataLL {
   public:
    CdataLL(particleContainer &_ps, CglobalVars &_globals, sphdem_handle _h)
        : globals(_globals), ps(_ps), h(_h) {}

    CglobalVars &globals;

    /* the particle container, as a pointer as the reference returns it (dataLL.h:237-238) */
    particleContainer *getParticles() { return &ps; }
    sphdem_handle handle() const { return h; }

    /* device -> mirror (all fields, globals); neighbour lists on demand */
    void pull();
    /* mirror -> device (mutable fields, globals, deletions, insertions) */
    void push();

    /* CdataLL::insertNewParticle (dataLL.cpp:238-261) */
    void insertNewParticle(Cparticle &newP) { pending_insert.push_back(newP); }
    /* CdataLL::markForDeletion (dataLL.cpp:263-266) */
    void markForDeletion(Cparticle &p) { p.tag = -111; }
    /* CdataLL::deleteParticles (dataLL.cpp:272-283): marked particles leave at
     * the device's next rebuild, which every neighbour pass follows */
    void deleteParticles() {}

    template <void Thefunct(Cparticle &, CglobalVars &)>
    void traverse() {
        for (size_t i = 0; i < ps.size(); i++) Thefunct(ps[i], globals);
    }
    template <void Thefunct(Cparticle &, CglobalVars &), bool Iffunct(Cparticle &)>
    void traverse() {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], globals);
    }
    template <void Thefunct(Cparticle &, CglobalVars &, double)>
    void traverse(double a) {
        for (size_t i = 0; i < ps.size(); i++) Thefunct(ps[i], globals, a);
    }
    template <void Thefunct(Cparticle &, CglobalVars &, double), bool Iffunct(Cparticle &)>
    void traverse(double a) {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], globals, a);
    }
    template <void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &)>
    void neighboursGroup() {
        lists();
        for (size_t i = 0; i < ps.size(); i++) Thefunct(ps[i], nbrs[i], globals);
    }
    template <void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &), bool Iffunct(Cparticle &)>
    void neighboursGroup() {
        lists();
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], nbrs[i], globals);
    }

    /* the remaining traverse forms of dataLL.h:125-142 */
    template <class T, void Thefunct(Cparticle &, CglobalVars &, T &)>
    void traverse(T &a) {
        for (size_t i = 0; i < ps.size(); i++) Thefunct(ps[i], globals, a);
    }
    template <class T, void Thefunct(Cparticle &, CglobalVars &, T &), bool Iffunct(Cparticle &)>
    void traverse(T &a) {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], globals, a);
    }
    template <void Thefunct(Cparticle &, CglobalVars &, double, double)>
    void traverse(double a, double b) {
        for (size_t i = 0; i < ps.size(); i++) Thefunct(ps[i], globals, a, b);
    }
    template <void Thefunct(Cparticle &, CglobalVars &, double, double), bool Iffunct(Cparticle &)>
    void traverse(double a, double b) {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], globals, a, b);
    }
    template <void Thefunct(Cparticle &, CglobalVars &, double, double, double), bool Iffunct(Cparticle &)>
    void traverse(double a, double b, double c) {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], globals, a, b, c);
    }

    /* every (particle, neighbour) pair, in both orders (dataLL.impl.h:182-216) */
    template <void Thefunct(Cparticle &, Cparticle &, CglobalVars &)>
    void neighbours() {
        lists();
        for (size_t i = 0; i < ps.size(); i++)
            for (Cparticle *pn : nbrs[i]) Thefunct(ps[i], *pn, globals);
    }
    template <void Thefunct(Cparticle &, Cparticle &, CglobalVars &), bool Iffunct(Cparticle &)>
    void neighbours() {
        lists();
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i]))
                for (Cparticle *pn : nbrs[i]) Thefunct(ps[i], *pn, globals);
    }
    template <class T, void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &, T &), bool Iffunct(Cparticle &)>
    void neighboursGroup(T &a) {
        lists();
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], nbrs[i], globals, a);
    }

    /* neighbours of particles that are not in the simulation, e.g. points of
     * an output grid (dataLL.impl.h:283-306): the simulation's particles of
     * the query's relation (DEM for a DEM query, else the others) within
     * 2 max(h) of it, periodic images as ghost copies.  A search over all
     * particles per query, for output steps. */
    template <void Thefunct(Cparticle &, Cparticle &, CglobalVars &)>
    void neighboursUsing(vector<Cparticle> &qs) {
        for (Cparticle &q : qs) {
            vector<Cparticle *> found;
            search(q, -1.0, found);
            for (Cparticle *pn : found) Thefunct(q, *pn, globals);
        }
    }
    template <void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &)>
    void neighboursUsing(vector<Cparticle> &qs) {
        for (Cparticle &q : qs) {
            vector<Cparticle *> found;
            search(q, -1.0, found);
            Thefunct(q, found, globals);
        }
    }
    /* neighbours within a given radius (dataLL.impl.h:244-255), searched as
     * neighboursUsing searches */
    template <void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &), bool Iffunct(Cparticle &)>
    void neighboursGroupAtRadius(const double radius) {
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) {
                vector<Cparticle *> found;
                search(ps[i], radius, found);
                Thefunct(ps[i], found, globals);
            }
    }

#ifdef LIQ_DEM
    /* the coupling neighbours (dataLL.impl.h:257-268, calcNeighboursCoupling
     * dataLL.cpp:1104-1192): a fluid particle's DEM particles under the
     * reference's coupling bucket rule, a DEM particle's SPH-grid neighbours,
     * periodic partners as ghost copies at their nearest image */
    template <void Thefunct(Cparticle &, vector<Cparticle *> &, CglobalVars &), bool Iffunct(Cparticle &)>
    void neighboursGroupCoupling() {
        coupling_lists();
        for (size_t i = 0; i < ps.size(); i++)
            if (Iffunct(ps[i])) Thefunct(ps[i], cnbrs[i], globals);
    }
#endif

    int numParticles() { return (int)ps.size(); }
    /* CdataLL::reset (dataLL.cpp:140-236) from case code: the mirror's state
     * goes to the device, which rebuilds its buckets and lists there, and
     * comes back */
    void reset() {
        push();
        check(sphdem_rebuild(h), "sphdem_rebuild");
        pull();
    }
    /* CdataLL::sumOverProcs (dataLL.cpp:790-830): one process holds every
     * particle, so the sums are the values themselves */
    void sumOverProcs(vect *, int) {}
    void sumOverProcs(double *, int) {}

   private:
    particleContainer &ps;
    sphdem_handle h;
    vector<Cparticle> pending_insert;
    vector<vector<Cparticle *> > nbrs, cnbrs;
    /* periodic images of neighbours: copies with the position shifted by a
     * period, as the reference's ghost particles are (dataLL.cpp:648-660);
     * pointers stay valid while the deque grows */
    std::deque<Cparticle> ghosts;
    std::unordered_map<long long, Cparticle *> ghost_of; /* (particle, shift) -> its ghost */
    bool lists_valid = false, clists_valid = false;
    vector<double> vu, vdudt, vev, vdev;
    vector<double> vr, vv, vvh, vv0, vvh0, vf, vfp, vfv, vfb, vfd, vfvel, vgp, vn1, vn2, vn3;
    vector<double> vm, vd, vh, vrad, vdddt, vpress, vpdr2, vpor, vdpor, vshep, vom;
    vector<int32_t> viam, vtag;
    vector<uint8_t> vconc;

    void check(int rc, const char *what) {
        if (rc == SPHDEM_OK) return;
        char msg[512];
        sphdem_last_error(h, msg, sizeof msg);
        std::cerr << what << ": " << msg << std::endl;
        std::exit(-1); /* the reference's error behaviour */
    }
    void soa(SphDemParticles &p);
    void lists();
    void coupling_lists();
    /* one relation of the device as CSR over tag order */
    void relation(int kind, vector<int64_t> &offs, vector<int32_t> &idx);
    Cparticle *image_of(Cparticle &q, Cparticle &b);
    Cparticle *ghost(Cparticle &b, const int *shift);
    void search(Cparticle &q, double radius, vector<Cparticle *> &found);
};

inline void CdataLL::soa(SphDemParticles &p) {
    const size_t n = ps.size();
    auto v3 = [n](vector<double> &v) { v.resize(3 * n); return v.data(); };
    auto v1 = [n](vector<double> &v) { v.resize(n); return v.data(); };
    std::memset(&p, 0, sizeof p);
    p.n = (int64_t)n;
    viam.resize(n);
    vtag.resize(n);
    vconc.resize(n);
    p.iam = viam.data();
    p.tag = vtag.data();
    p.concave = vconc.data();
    p.r = v3(vr); p.v = v3(vv); p.vhat = v3(vvh); p.v0 = v3(vv0); p.vhat0 = v3(vvh0);
    p.f = v3(vf); p.fp = v3(vfp); p.fv = v3(vfv); p.fb = v3(vfb);
    p.fdrag = v3(vfd); p.fvel = v3(vfvel); p.grad_porosity = v3(vgp);
    p.norm1 = v3(vn1); p.norm2 = v3(vn2); p.norm3 = v3(vn3);
    p.mass = v1(vm); p.dens = v1(vd); p.h = v1(vh); p.radius = v1(vrad); p.dddt = v1(vdddt);
    p.press = v1(vpress); p.pdr2 = v1(vpdr2); p.porosity = v1(vpor); p.dporositydt = v1(vdpor);
    p.shep_sum = v1(vshep); p.omega = v1(vom);
    p.u = v1(vu); p.dudt = v1(vdudt); p.e_visc = v1(vev); p.de_visc_dt = v1(vdev);
}

inline void CdataLL::pull() {
    SphDemParticles p;
    soa(p);
    check(sphdem_get_fields(h, SPHDEM_FIELD_ALL, &p), "sphdem_get_fields");
    for (size_t i = 0; i < ps.size(); i++) {
        Cparticle &q = ps[i];
        for (int d = 0; d < NDIM; d++) {
            q.r[d] = vr[3 * i + d]; q.v[d] = vv[3 * i + d]; q.vhat[d] = vvh[3 * i + d];
            q.v0[d] = vv0[3 * i + d]; q.vhat0[d] = vvh0[3 * i + d];
            q.f[d] = vf[3 * i + d]; q.fp[d] = vfp[3 * i + d]; q.fv[d] = vfv[3 * i + d]; q.fb[d] = vfb[3 * i + d];
            q.fdrag[d] = vfd[3 * i + d]; q.fvel[d] = vfvel[3 * i + d]; q.gradPorosity[d] = vgp[3 * i + d];
            q.norm1[d] = vn1[3 * i + d]; q.norm2[d] = vn2[3 * i + d]; q.norm3[d] = vn3[3 * i + d];
        }
        q.mass = vm[i]; q.dens = vd[i]; q.h = vh[i]; q.radius = vrad[i]; q.dddt = vdddt[i];
        q.press = vpress[i]; q.pdr2 = vpdr2[i]; q.porosity = vpor[i]; q.dporositydt = vdpor[i];
        q.shepSum = vshep[i]; q.omega = vom[i];
        q.u = vu[i]; q.dudt = vdudt[i]; q.eViscF = vev[i]; q.deViscFdt = vdev[i];
        q.iam = (iamTypes)viam[i];
        q.tag = vtag[i];
        q.concave = vconc[i] != 0;
    }
    SphDemGlobals g;
    check(sphdem_get_globals(h, &g), "sphdem_get_globals");
    globals.time = g.time;
    globals.dt = g.dt;
    globals.newDt = g.new_dt;
    globals.maxdt = g.maxdt;
    globals.demDt = g.dem_dt;
    globals.sphStep = (int)g.sph_step;
    globals.n = (int)ps.size();
    /* neighbour lists and ghost copies follow the new state */
    lists_valid = false;
    clists_valid = false;
    ghosts.clear();
    ghost_of.clear();
}

inline void CdataLL::push() {
    /* buffers sized for the mirror first (it grows at insertions) */
    SphDemParticles p;
    soa(p);
    for (size_t i = 0; i < ps.size(); i++) {
        const Cparticle &q = ps[i];
        for (int d = 0; d < NDIM; d++) {
            vr[3 * i + d] = q.r[d]; vv[3 * i + d] = q.v[d]; vvh[3 * i + d] = q.vhat[d];
            vf[3 * i + d] = q.f[d]; vfp[3 * i + d] = q.fp[d]; vfv[3 * i + d] = q.fv[d]; vfb[3 * i + d] = q.fb[d];
        }
        vd[i] = q.dens;
        vh[i] = q.h;
    }
    check(sphdem_set_fields(h, SPHDEM_FIELD_R | SPHDEM_FIELD_V | SPHDEM_FIELD_VHAT | SPHDEM_FIELD_F |
                                   SPHDEM_FIELD_DENS | SPHDEM_FIELD_H, &p),
          "sphdem_set_fields");
    SphDemGlobals g;
    check(sphdem_get_globals(h, &g), "sphdem_get_globals");
    g.time = globals.time;
    g.maxdt = globals.maxdt;
    check(sphdem_set_globals(h, &g), "sphdem_set_globals");
    vector<int64_t> del;
    for (size_t i = 0; i < ps.size(); i++)
        if (ps[i].tag == -111 && viam[i] >= 0) del.push_back((int64_t)i);
    if (!del.empty()) check(sphdem_mark_for_deletion(h, del.data(), (int64_t)del.size()), "sphdem_mark_for_deletion");
    if (!pending_insert.empty()) {
        const size_t k = pending_insert.size();
        vector<int32_t> iam(k);
        vector<uint8_t> conc(k);
        vector<double> r(3 * k, 0.0), v(3 * k, 0.0), vh(3 * k, 0.0), n1(3 * k, 0.0), n2(3 * k, 0.0), n3(3 * k, 0.0);
        vector<double> m(k), d(k), hh(k), rad(k);
        for (size_t j = 0; j < k; j++) {
            const Cparticle &q = pending_insert[j];
            iam[j] = (int32_t)q.iam;
            conc[j] = q.concave ? 1 : 0;
            for (int a = 0; a < NDIM; a++) {
                r[3 * j + a] = q.r[a];
                v[3 * j + a] = q.v[a];
                vh[3 * j + a] = q.vhat[a];
                n1[3 * j + a] = q.norm1[a];
                n2[3 * j + a] = q.norm2[a];
                n3[3 * j + a] = q.norm3[a];
            }
            m[j] = q.mass;
            d[j] = q.dens;
            hh[j] = q.h;
            rad[j] = q.radius;
        }
        SphDemParticles in;
        std::memset(&in, 0, sizeof in);
        in.n = (int64_t)k;
        in.iam = iam.data(); in.concave = conc.data();
        in.r = r.data(); in.v = v.data(); in.vhat = vh.data();
        in.norm1 = n1.data(); in.norm2 = n2.data(); in.norm3 = n3.data();
        in.mass = m.data(); in.dens = d.data(); in.h = hh.data(); in.radius = rad.data();
        vector<int64_t> slot(k);
        check(sphdem_insert_particles(h, &in, slot.data()), "sphdem_insert_particles");
        size_t n = ps.size();
        for (int64_t s : slot) n = std::max(n, (size_t)s + 1);
        ps.resize(n);
        for (size_t j = 0; j < k; j++) ps[slot[j]] = pending_insert[j];
        pending_insert.clear();
        /* the container may have moved: lists and ghosts are rebuilt on use */
        lists_valid = false;
        clists_valid = false;
        ghosts.clear();
        ghost_of.clear();
    }
}

inline void CdataLL::lists() {
    if (lists_valid) return;
    const size_t n = ps.size();
    /* calcNeighbours (dataLL.cpp:1026-1075): DEM particles take the DEM
     * relation, the others the SPH one; each row comes from one of the two */
    vector<int64_t> offs[2];
    vector<int32_t> idx[2];
    relation(SPHDEM_PAIRS_SPH, offs[0], idx[0]);
    relation(SPHDEM_PAIRS_DEM, offs[1], idx[1]);
    nbrs.assign(n, vector<Cparticle *>());
    for (size_t i = 0; i < n; i++) {
        const int k = ps[i].iam == dem ? 1 : 0;
        for (int64_t e = offs[k][i]; e < offs[k][i + 1]; e++) nbrs[i].push_back(image_of(ps[i], ps[idx[k][e]]));
    }
    lists_valid = true;
}

inline void CdataLL::relation(int kind, vector<int64_t> &offs, vector<int32_t> &idx) {
    offs.assign(ps.size() + 1, 0);
    int64_t np = 0;
    check(sphdem_pairs(h, kind, offs.data(), nullptr, 0, &np), "sphdem_pairs");
    idx.resize((size_t)np);
    check(sphdem_pairs(h, kind, offs.data(), idx.data(), np, &np), "sphdem_pairs");
}

inline void CdataLL::coupling_lists() {
    if (clists_valid) return;
    const size_t n = ps.size();
    /* fluid -> DEM rows of sph / sphBoundary particles, DEM -> fluid rows of
     * DEM particles; each row comes from one of the two relations */
    vector<int64_t> offs[2];
    vector<int32_t> idx[2];
    relation(SPHDEM_PAIRS_COUPLE_SD, offs[0], idx[0]);
    relation(SPHDEM_PAIRS_COUPLE_DS, offs[1], idx[1]);
    cnbrs.assign(n, vector<Cparticle *>());
    for (size_t i = 0; i < n; i++) {
        const int k = ps[i].iam == dem ? 1 : 0;
        for (int64_t e = offs[k][i]; e < offs[k][i + 1]; e++) cnbrs[i].push_back(image_of(ps[i], ps[idx[k][e]]));
    }
    clists_valid = true;
}

/* b itself, or, where b is p's neighbour across a periodic boundary, the
 * ghost copy of b at its periodic image nearest p: r = RMIN - RMAX + r or
 * RMAX - RMIN + r on that axis, as dataLL.cpp:648-660 places ghosts.  A
 * periodic axis spans at least three buckets of 2 h_max, so the nearest
 * image is the neighbour. */
inline Cparticle *CdataLL::image_of(Cparticle &p, Cparticle &b) {
    int shift[NDIM];
    bool any = false;
    for (int d = 0; d < NDIM; d++) {
        shift[d] = 0;
        if (!PERIODIC[d]) continue;
        const double half = 0.5 * (RMAX[d] - RMIN[d]);
        const double dx = p.r[d] - b.r[d];
        if (dx > half) shift[d] = 1;
        if (dx < -half) shift[d] = -1;
        any = any || shift[d] != 0;
    }
    return any ? ghost(b, shift) : &b;
}

/* the ghost copy of particle b shifted by whole periods (shift[d] in
 * {-1, 0, 1}), one per particle and shift, as the reference keeps one ghost
 * particle per image */
inline Cparticle *CdataLL::ghost(Cparticle &b, const int *shift) {
    long long key = (long long)(&b - &ps[0]);
    for (int d = 0; d < NDIM; d++) key = 3 * key + (shift[d] + 1);
    auto it = ghost_of.find(key);
    if (it != ghost_of.end()) return it->second;
    ghosts.push_back(b);
    Cparticle &g = ghosts.back();
    for (int d = 0; d < NDIM; d++) {
        if (shift[d] > 0) g.r[d] = RMAX[d] - RMIN[d] + b.r[d];
        if (shift[d] < 0) g.r[d] = RMIN[d] - RMAX[d] + b.r[d];
    }
    ghost_of[key] = &g;
    return &g;
}

/* every particle of q's relation (DEM for a DEM query, else the others)
 * whose nearest image lies within 2 max(h) of q (radius < 0) or within
 * radius, the image as a ghost copy where it is not the particle itself */
inline void CdataLL::search(Cparticle &q, double radius, vector<Cparticle *> &found) {
    const bool dem_q = q.iam == dem;
    for (size_t j = 0; j < ps.size(); j++) {
        Cparticle &b = ps[j];
        if (&b == &q || (b.iam == dem) != dem_q || (int)b.iam < 0) continue;
        Cparticle *img = image_of(q, b);
        const double lim2 = radius < 0 ? std::pow(2.0 * (q.h > b.h ? q.h : b.h), 2) : radius * radius;
        if (len2(q.r - img->r) <= lim2) found.push_back(img);
    }
}

#endif
