/*
 * Driver for the reference's own hot path, compiled from the unmodified
 * reference sources as a CPU checker (test infrastructure only).
 *
 * It stands in for the reference's `setup` + `run` executables without VTK:
 * it reads a seeded initial state (SPDMST01, written by the case generators),
 * builds CdataLL/CsphIncompress/CcustomSim exactly as run.cpp:80-83 does, runs
 * the step loop of run.cpp:102-119 and writes every hot-path field, the
 * neighbour relations and the bucket indices in tag order (SPDMOUT1).
 *
 * Usage: ref_driver <in.state> <out.bin> <nsteps> [timing-only(0|1)]
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <list>
#include <sstream>
#include <string>
#include <sys/time.h>
#include <vector>

/* Internals of CdataLL (bucket maps, cells) are read for the dump only. */
#define private public
#include "customConstants.h"
#include "sphIncompress.h"
#include "customSim.h"
#include "misc.h"
#undef private

/* misc.cpp refers to these two writers; the checker writes no VTK. */
void Cio_data_vtk::writeAux(int, particleContainer &, vector<double>, const char *, CglobalVars *) {}
void Cio_data_vtk::writeAuxNoData(int, particleContainer &, const char *, CglobalVars *) {}

static void fail(const char *msg) {
    fprintf(stderr, "ref_driver: %s\n", msg);
    exit(2);
}

template <class T>
static void rd(std::ifstream &in, T *p, size_t n) {
    in.read(reinterpret_cast<char *>(p), sizeof(T) * n);
    if (!in) fail("short read");
}

struct Field {
    std::string name;
    int ncomp;
    std::vector<double> data;
};

/* particle arrays of the state file (tag order) */
struct Block {
    std::vector<int> iam, tag, concave;
    std::vector<double> r, v, mass, dens, h, radius, n1, n2, n3;
};

static void read_block(std::ifstream &in, long long n, bool with_tag, Block &b) {
    b.iam.resize(n);
    b.tag.resize(n);
    b.concave.resize(n);
    b.r.resize(3 * n);
    b.v.resize(3 * n);
    b.mass.resize(n);
    b.dens.resize(n);
    b.h.resize(n);
    b.radius.resize(n);
    b.n1.resize(3 * n);
    b.n2.resize(3 * n);
    b.n3.resize(3 * n);
    rd(in, b.iam.data(), n);
    if (with_tag) rd(in, b.tag.data(), n);
    rd(in, b.concave.data(), n);
    rd(in, b.r.data(), 3 * n);
    rd(in, b.v.data(), 3 * n);
    rd(in, b.mass.data(), n);
    rd(in, b.dens.data(), n);
    rd(in, b.h.data(), n);
    rd(in, b.radius.data(), n);
    rd(in, b.n1.data(), 3 * n);
    rd(in, b.n2.data(), 3 * n);
    rd(in, b.n3.data(), 3 * n);
}

static Cparticle to_particle(const Block &b, long long i, int tag) {
    Cparticle p;
    p.iam = (enum iamTypes)b.iam[i];
    p.tag = tag;
    p.concave = b.concave[i] != 0;
    for (int d = 0; d < NDIM; d++) {
        p.r[d] = b.r[3 * i + d];
        p.v[d] = b.v[3 * i + d];
        p.norm1[d] = b.n1[3 * i + d];
        p.norm2[d] = b.n2[3 * i + d];
#ifdef _3D_
        p.norm3[d] = b.n3[3 * i + d];
#endif
    }
    p.vhat = p.v;
    p.mass = b.mass[i];
    p.dens = b.dens[i];
    p.h = b.h[i];
    /* members the Cparticle constructor leaves unset (particle.h:67-131) and
     * the step never writes for every type: zero, as in fresh memory */
    p.deViscFdt = 0.0;
    p.fb = 0.0;
    p.ff = 0.0;
    return p;
}

/* one scheduled change: insert a block (kind 1) or mark tag-order indices
 * for deletion (kind 2) */
struct Event {
    long long step = 0;
    int kind = 0;
    Block add;
    std::vector<long long> del;
};

static void put_name(FILE *f, const std::string &s) {
    char buf[16];
    memset(buf, 0, 16);
    strncpy(buf, s.c_str(), 15);
    fwrite(buf, 1, 16, f);
}

int main(int argc, char **argv) {
    if (argc < 4) fail("usage: ref_driver in out nsteps [timing-only]");
    const int nsteps = atoi(argv[3]);
    const bool timing_only = argc > 4 && atoi(argv[4]) != 0;

    std::ifstream in(argv[1], std::ios::binary);
    if (!in) fail("cannot open input");
    char magic[8];
    rd(in, magic, 8);
    if (memcmp(magic, "SPDMST01", 8) != 0) fail("bad magic");
    long long n;
    rd(in, &n, 1);
    Block init;
    read_block(in, n, true, init);

    /* optional schedule of insertions and deletions (SPDMEV01), applied
     * after afterEnd of their step as a case's own afterEnd hook would */
    std::vector<Event> events;
    if (in.peek() != EOF) {
        rd(in, magic, 8);
        if (memcmp(magic, "SPDMEV01", 8) != 0) fail("bad event magic");
        long long ne;
        rd(in, &ne, 1);
        events.resize(ne);
        for (long long e = 0; e < ne; e++) {
            long long hdr[3];
            rd(in, hdr, 3);
            events[e].step = hdr[0];
            events[e].kind = (int)hdr[1];
            if (events[e].kind == 1) {
                read_block(in, hdr[2], false, events[e].add);
            } else if (events[e].kind == 2) {
                events[e].del.resize(hdr[2]);
                rd(in, events[e].del.data(), hdr[2]);
            } else {
                fail("bad event kind");
            }
        }
    }

    vector<Cparticle> ps;
    ps.reserve(std::max<long long>(MAX_NUM_PARTICLES_PER_CPU, n + 64));
    for (long long i = 0; i < n; i++) ps.push_back(to_particle(init, i, init.tag[i]));

    CglobalVars g;
    Nmisc::setupEntireDomain(g.procDomain, g.procNeighbrs);
    g.maxdt = ORACLE_MAXDT;
    g.dt = ORACLE_MAXDT;
    /* The O(N^2) insertion sort of the initial traverse order
     * (dataLL.cpp:887-904) only sets the visit order; skip it for big runs. */
    CdataLL *data = new CdataLL(ps, g, n <= 20000);
    CsphIncompress solver(data);
    CcustomSim customSim(data, g.time);

    int dt_changed = 0;
    long long ntot = n;          /* tags handed out so far */
    std::vector<int> pending;    /* tags marked for deletion, not yet deleted */
    timeval t0, t1;
    gettimeofday(&t0, NULL);
    for (int k = 0; k < nsteps; k++) {
        g.sphStep++;
        customSim.beforeStart(g.time);
        solver.start();
        customSim.beforeMiddle(g.time);
        solver.middle();
        customSim.beforeEnd(g.time);
        solver.end();
        customSim.afterEnd(g.time);
        if (g.dt != ORACLE_MAXDT) dt_changed++;
        for (const Event &ev : events) {
            if (ev.step != g.sphStep) continue;
            /* a marked particle (tag -111) keeps its slot until the reset
             * that deletes it */
            bool marked_present = false;
            for (const Cparticle &p : ps) marked_present |= p.tag == -111;
            if (!marked_present) pending.clear();
            if (ev.kind == 2) {
                for (long long idx : ev.del) {
                    bool found = false;
                    for (Cparticle &p : ps)
                        if (p.tag == idx + 1) {
                            data->markForDeletion(p);
                            found = true;
                            break;
                        }
                    if (!found) fail("deletion of a particle that is not there");
                    pending.push_back((int)idx + 1);
                }
            } else {
                /* tags in the library's slot order: the lowest free tag, else the next */
                std::vector<char> used(ntot + 2 + ev.add.iam.size(), 0);
                for (const Cparticle &p : ps)
                    if (p.tag >= 1) used[p.tag] = 1;
                for (int t : pending) used[t] = 1;
                long long cursor = 1;
                for (size_t i = 0; i < ev.add.iam.size(); i++) {
                    while (cursor <= ntot && used[cursor]) cursor++;
                    long long t;
                    if (cursor <= ntot) {
                        t = cursor;
                        used[cursor] = 1;
                    } else {
                        t = ++ntot;
                        cursor = ntot + 1;
                    }
                    Cparticle p = to_particle(ev.add, (long long)i, (int)t);
                    data->insertNewParticle(p);
                }
            }
        }
    }
    gettimeofday(&t1, NULL);
    const double sec = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
    fprintf(stderr, "ref_driver: n=%zu steps=%d sec=%.6f particle_steps_per_s=%.6e dt_changed=%d\n",
            ps.size(), nsteps, sec, ps.size() * (double)nsteps / (sec > 0 ? sec : 1e-30), dt_changed);
    /* a fixed-dt case must keep the reference's adaptive dt at maxdt */
    if (timing_only) return (ORACLE_FIXED_DT && dt_changed) ? 3 : 0;

    /* tag -> position in ps (periodic exchange reorders ps); a tag without a
     * particle was deleted and is written as zeros with alive = 0 */
    n = ntot;
    std::vector<long long> row_of_tag(n + 1, -1);
    for (size_t i = 0; i < ps.size(); i++) {
        if (ps[i].tag < 1 || ps[i].tag > n) fail("tag out of range");
        row_of_tag[ps[i].tag] = i;
    }
    if (events.empty())
        for (long long t = 1; t <= n; t++)
            if (row_of_tag[t] < 0) fail("particle lost (deleted?)");

    std::vector<Field> fields;
    auto vec_field = [&](const char *name, vect Cparticle::*m) {
        Field f{name, 3, std::vector<double>(3 * n, 0.0)};
        for (long long t = 1; t <= n; t++) {
            if (row_of_tag[t] < 0) continue;
            const Cparticle &p = ps[row_of_tag[t]];
            for (int d = 0; d < NDIM; d++) f.data[3 * (t - 1) + d] = (p.*m)[d];
        }
        fields.push_back(f);
    };
    auto sca_field = [&](const char *name, double Cparticle::*m) {
        Field f{name, 1, std::vector<double>(n, 0.0)};
        for (long long t = 1; t <= n; t++)
            if (row_of_tag[t] >= 0) f.data[t - 1] = ps[row_of_tag[t]].*m;
        fields.push_back(f);
    };
    {
        Field f{"alive", 1, std::vector<double>(n, 0.0)};
        for (long long t = 1; t <= n; t++) f.data[t - 1] = row_of_tag[t] >= 0 ? 1.0 : 0.0;
        fields.push_back(f);
    }
    vec_field("r", &Cparticle::r);
    vec_field("v", &Cparticle::v);
    vec_field("vhat", &Cparticle::vhat);
    vec_field("v0", &Cparticle::v0);
    vec_field("vhat0", &Cparticle::vhat0);
    vec_field("f", &Cparticle::f);
    vec_field("fp", &Cparticle::fp);
    vec_field("fv", &Cparticle::fv);
    vec_field("fb", &Cparticle::fb);
    sca_field("dens", &Cparticle::dens);
    sca_field("dddt", &Cparticle::dddt);
    sca_field("h", &Cparticle::h);
    sca_field("press", &Cparticle::press);
    sca_field("pdr2", &Cparticle::pdr2);
    sca_field("mass", &Cparticle::mass);
    sca_field("u", &Cparticle::u);
    sca_field("dudt", &Cparticle::dudt);
    sca_field("eViscF", &Cparticle::eViscF);
    sca_field("deViscFdt", &Cparticle::deViscFdt);
#ifdef LIQ_DEM
    sca_field("porosity", &Cparticle::porosity);
    sca_field("dporositydt", &Cparticle::dporositydt);
    vec_field("gradPorosity", &Cparticle::gradPorosity);
    sca_field("shepSum", &Cparticle::shepSum);
    vec_field("fdrag", &Cparticle::fdrag);
    vec_field("fvel", &Cparticle::fvel);
#endif
#ifdef VAR_H_CORRECTION
    sca_field("omega", &Cparticle::omega);
#endif

    /* the output-step globals, as run.cpp:131 computes them (on the cached
     * lists of the last reset) */
    solver.calcOutputVars();
    std::vector<double> ov;
    for (int d = 0; d < 3; d++) ov.push_back(d < NDIM ? g.linMom[d] : 0.0);
    const double ovs[] = {g.angMom, g.eKE, g.eElast, g.eElastExact, g.edElastdt, g.eViscF, g.edViscFdt,
                          g.eFF, g.edFFdt, g.eViscB, g.eBForce, g.eTotal, g.maxV, g.maxF, g.maxFF, g.rmsFF,
                          g.aveDens, g.varDens, g.aveDensFromMass, (double)g.n, (double)g.nSph};
    for (double x : ovs) ov.push_back(x);

    /* neighbour relations at the final positions, after one more reset so
     * that the ghost copies carry the smoothing lengths driftRest just
     * updated -- exactly the lists the next traversal would build
     * (dataLL.cpp:1026-1075, 1104-1192) */
    data->reset();
    struct Rel { std::string name; std::vector<std::vector<int> > rows; };
    std::vector<Rel> rels;
    Rel sphrel{"sph", std::vector<std::vector<int> >(n)};
    Rel demrel{"dem", std::vector<std::vector<int> >(n)};
    Rel sdrel{"couple_sd", std::vector<std::vector<int> >(n)};
    Rel dsrel{"couple_ds", std::vector<std::vector<int> >(n)};
    int duplicates = 0;
    /* the reset moved particles: map tags again */
    std::fill(row_of_tag.begin(), row_of_tag.end(), -1);
    for (size_t i = 0; i < ps.size(); i++)
        if (ps[i].tag >= 1 && ps[i].tag <= n) row_of_tag[ps[i].tag] = i;
    for (long long t = 1; t <= n; t++) {
        if (row_of_tag[t] < 0) continue;
        Cparticle &p = ps[row_of_tag[t]];
        std::vector<Cparticle *> nb;
        data->calcNeighbours(nb, p);
        std::vector<int> &row = (p.iam == dem) ? demrel.rows[t - 1] : sphrel.rows[t - 1];
        for (size_t j = 0; j < nb.size(); j++) row.push_back(nb[j]->tag - 1);
#ifdef LIQ_DEM
        std::vector<Cparticle *> cn;
        data->calcNeighboursCoupling(cn, p);
        if (p.iam == dem) {
            for (size_t j = 0; j < cn.size(); j++) dsrel.rows[t - 1].push_back(cn[j]->tag - 1);
        } else if (p.iam == sph || p.iam == sphBoundary) {
            for (size_t j = 0; j < cn.size(); j++)
                if (len2(p.r - cn[j]->r) < pow(LIQ_DEM_COUPLING_RADIUS, 2))
                    sdrel.rows[t - 1].push_back(cn[j]->tag - 1);
        }
#endif
    }
    rels.push_back(sphrel);
    rels.push_back(demrel);
#ifdef LIQ_DEM
    rels.push_back(sdrel);
    rels.push_back(dsrel);
#endif
    for (size_t k = 0; k < rels.size(); k++)
        for (long long i = 0; i < n; i++) {
            std::vector<int> &row = rels[k].rows[i];
            std::sort(row.begin(), row.end());
            size_t before = row.size();
            row.erase(std::unique(row.begin(), row.end()), row.end());
            duplicates += (int)(before - row.size());
        }
    if (duplicates) fprintf(stderr, "ref_driver: warning: %d duplicate neighbour entries (periodic images)\n", duplicates);

    FILE *out = fopen(argv[2], "wb");
    if (!out) fail("cannot open output");
    fwrite("SPDMOUT1", 1, 8, out);
    fwrite(&n, 8, 1, out);
    long long nf = fields.size();
    fwrite(&nf, 8, 1, out);
    for (size_t k = 0; k < fields.size(); k++) {
        put_name(out, fields[k].name);
        long long nc = fields[k].ncomp;
        fwrite(&nc, 8, 1, out);
        fwrite(fields[k].data.data(), 8, fields[k].data.size(), out);
    }
    long long nk = rels.size();
    fwrite(&nk, 8, 1, out);
    for (size_t k = 0; k < rels.size(); k++) {
        put_name(out, rels[k].name);
        std::vector<long long> offs(n + 1, 0);
        for (long long i = 0; i < n; i++) offs[i + 1] = offs[i] + rels[k].rows[i].size();
        long long np = offs[n];
        fwrite(&np, 8, 1, out);
        fwrite(offs.data(), 8, n + 1, out);
        for (long long i = 0; i < n; i++)
            if (!rels[k].rows[i].empty()) fwrite(rels[k].rows[i].data(), 4, rels[k].rows[i].size(), out);
    }
    std::vector<int> cells(3 * n, 0);
    for (long long t = 1; t <= n; t++) {
        if (row_of_tag[t] < 0) continue;
        Cparticle &p = ps[row_of_tag[t]];
        vectInt c;
#ifdef LIQ_DEM
        if (p.iam == dem) c = data->dem_getCellI(p.r); else
#endif
        c = data->getCellI(p.r);
        for (int d = 0; d < NDIM; d++) cells[3 * (t - 1) + d] = c[d];
    }
    fwrite(cells.data(), 4, 3 * n, out);
    double tt[2] = {g.time, g.dt};
    fwrite(tt, 8, 2, out);
    /* trailer: the calcOutputVars globals (order of SphDemOutputVars) */
    long long nov = ov.size();
    fwrite(&nov, 8, 1, out);
    fwrite(ov.data(), 8, ov.size(), out);
    fclose(out);
    return (ORACLE_FIXED_DT && dt_changed) ? 3 : 0;
}
