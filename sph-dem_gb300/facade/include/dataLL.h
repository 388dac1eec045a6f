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
#include <iostream>
#include <string>
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

    particleContainer &getParticles() { return ps; }
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

   private:
    particleContainer &ps;
    sphdem_handle h;
    vector<Cparticle> pending_insert;
    vector<vector<Cparticle *> > nbrs;
    bool lists_valid = false;
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
    lists_valid = false;
}

inline void CdataLL::push() {
    for (size_t i = 0; i < ps.size(); i++) {
        const Cparticle &q = ps[i];
        for (int d = 0; d < NDIM; d++) {
            vr[3 * i + d] = q.r[d]; vv[3 * i + d] = q.v[d]; vvh[3 * i + d] = q.vhat[d];
            vf[3 * i + d] = q.f[d]; vfp[3 * i + d] = q.fp[d]; vfv[3 * i + d] = q.fv[d]; vfb[3 * i + d] = q.fb[d];
        }
        vd[i] = q.dens;
        vh[i] = q.h;
    }
    SphDemParticles p;
    soa(p);
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
        lists_valid = false;
    }
}

inline void CdataLL::lists() {
    if (lists_valid) return;
    const size_t n = ps.size();
    vector<int64_t> offs(n + 1);
    int64_t np = 0;
    check(sphdem_pairs(h, SPHDEM_PAIRS_SPH, offs.data(), nullptr, 0, &np), "sphdem_pairs");
    vector<int32_t> idx((size_t)np);
    check(sphdem_pairs(h, SPHDEM_PAIRS_SPH, offs.data(), idx.data(), np, &np), "sphdem_pairs");
    nbrs.assign(n, vector<Cparticle *>());
    for (size_t i = 0; i < n; i++)
        for (int64_t k = offs[i]; k < offs[i + 1]; k++) nbrs[i].push_back(&ps[idx[k]]);
    lists_valid = true;
}

#endif
