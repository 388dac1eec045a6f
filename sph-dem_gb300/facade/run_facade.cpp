/*
 * Driver of a case directory on the device (the step loop of run.cpp:16-164):
 * compiled together with the case's customConstants.h, customSim.cpp and
 * customOutput.cpp against the façade headers (include/), linked with
 * libsphdem.so.  Two command lines:
 *
 *   run_case <inbase> <intimestep> <outbase> [--mixed] [--fixed-dt]
 *
 * is run.cpp's own (used when <inbase> is not a file): the Domain, Globals
 * row and restart piece of output step <intimestep> are read from
 * <inbase>Domain0.dat, <inbase>Globals0.dat and
 * <inbase>Restart%07d_0.vtu; then, as run.cpp does, the case's hooks and
 * the device phases step while time <= MAXTIME and the output step <=
 * OUTSTEP, with maxdt = MAXTIME / OUTSTEP, and every MAXTIME / OUTSTEP of
 * simulated time come the output-step diagnostics, the case's calcOutput,
 * <outbase>%07d output pieces and a Globals row, and every
 * RESTART_EVERY_N_STEPS output steps a restart and a Domain file.
 * TIME_OVERIDE / START_TIME, NSTEP_OVERIDE / START_NSTEP and
 * START_WRITE_TIME apply as in run.cpp when the case defines them.
 *
 *   run_case <initial state> <nsteps> <final state out> [--mixed] [--fixed-dt]
 *            [--restart-out <base>] [--dump-config <file>]
 *
 * runs a fixed number of steps from a state file: a restart piece or index
 * (<base>Restart0000000_0.vtu / .pvtu, read as Cio_data_vtk::readRestart
 * reads it) or an SPDMST01 state file, with calcOutput every OUTSTEP steps.
 * The final state is written as r, v, vhat, f, dens, h per particle (tag
 * order) after a 16-byte header ("SPDMFAC1", n).  --restart-out writes it
 * also as <base>Restart%07d (the step count) with Float64 points;
 * --dump-config writes the SphDemConfig the case's constants give (raw
 * struct bytes).
 *
 * Every step calls the case's beforeStart / beforeMiddle / beforeEnd /
 * afterEnd hooks on the host mirror between the device phases
 * (SPHDEM_PHASE_START / MIDDLE / END).
 */
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "customConstants.h"
#include "customOutput.h"
#include "customSim.h"
#include "io_data_vtk.h"
#include "sphdem_case_config.h"

namespace {

bool ends_with(const std::string &s, const char *suf) {
    const size_t k = std::strlen(suf);
    return s.size() >= k && s.compare(s.size() - k, k, suf) == 0;
}

/* the SphDemParticles view of particles read from a restart, in tag order */
void soa_of(particleContainer &ps, SphDemParticles &p, std::vector<std::vector<char> > &keep);

/* a .vtu piece or a .pvtu index (its pieces in order) -> particles, then the
 * SphDemParticles view of them, in tag order */
bool read_vtk_state(const std::string &path, SphDemParticles &p, std::vector<std::vector<char> > &keep) {
    particleContainer ps;
    if (ends_with(path, ".pvtu")) {
        std::ifstream in(path.c_str());
        std::string line, dir = path.substr(0, path.find_last_of('/') + 1);
        while (std::getline(in, line)) {
            const size_t at = line.find("<Piece Source=\"");
            if (at == std::string::npos) continue;
            const size_t b = at + 15, e = line.find('"', b);
            particleContainer part;
            if (!Cio_data_vtk::readPiece(dir + line.substr(b, e - b), part)) return false;
            ps.insert(ps.end(), part.begin(), part.end());
        }
    } else if (!Cio_data_vtk::readPiece(path, ps)) {
        return false;
    }
    soa_of(ps, p, keep);
    return true;
}

void soa_of(particleContainer &ps, SphDemParticles &p, std::vector<std::vector<char> > &keep) {
    std::stable_sort(ps.begin(), ps.end(), [](const Cparticle &a, const Cparticle &b) { return a.tag < b.tag; });
    const int64_t n = (int64_t)ps.size();
    auto f64 = [&](size_t k) {
        keep.emplace_back(k * sizeof(double));
        return reinterpret_cast<double *>(keep.back().data());
    };
    auto i32 = [&]() {
        keep.emplace_back(n * sizeof(int32_t));
        return reinterpret_cast<int32_t *>(keep.back().data());
    };
    std::memset(&p, 0, sizeof p);
    p.n = n;
    p.iam = i32();
    p.tag = i32();
    keep.emplace_back(n);
    p.concave = reinterpret_cast<uint8_t *>(keep.back().data());
    p.r = f64(3 * n);
    p.v = f64(3 * n);
    p.vhat = f64(3 * n);
    p.norm1 = f64(3 * n);
    p.norm2 = f64(3 * n);
    p.norm3 = f64(3 * n);
    p.mass = f64(n);
    p.dens = f64(n);
    p.h = f64(n);
    p.radius = f64(n);
    for (int64_t i = 0; i < n; i++) {
        const Cparticle &q = ps[i];
        p.iam[i] = (int32_t)q.iam;
        p.tag[i] = (int32_t)i;
        p.concave[i] = 1;
        for (int d = 0; d < 3; d++) {
            p.r[3 * i + d] = d < NDIM ? q.r[d] : 0.0;
            p.v[3 * i + d] = d < NDIM ? q.v[d] : 0.0;
            p.vhat[3 * i + d] = d < NDIM ? q.vhat[d] : 0.0;
            p.norm1[3 * i + d] = d < NDIM ? q.norm1[d] : 0.0;
            p.norm2[3 * i + d] = d < NDIM ? q.norm2[d] : 0.0;
            p.norm3[3 * i + d] = d < NDIM ? q.norm3[d] : 0.0;
        }
        p.mass[i] = q.mass;
        p.dens[i] = q.dens;
        p.h[i] = q.h;
        p.radius[i] = q.radius;
    }
}

bool read_state(const char *path, SphDemParticles &p, std::vector<std::vector<char> > &keep) {
    std::ifstream in(path, std::ios::binary);
    char magic[8];
    if (!in.read(magic, 8) || std::memcmp(magic, "SPDMST01", 8) != 0) return false;
    int64_t n = 0;
    in.read(reinterpret_cast<char *>(&n), 8);
    auto take = [&](size_t bytes) -> char * {
        keep.emplace_back(bytes);
        in.read(keep.back().data(), (std::streamsize)bytes);
        return keep.back().data();
    };
    std::memset(&p, 0, sizeof p);
    p.n = n;
    p.iam = reinterpret_cast<int32_t *>(take(4 * n));
    p.tag = reinterpret_cast<int32_t *>(take(4 * n));
    int32_t *conc = reinterpret_cast<int32_t *>(take(4 * n));
    keep.emplace_back(n);
    p.concave = reinterpret_cast<uint8_t *>(keep.back().data());
    for (int64_t i = 0; i < n; i++) p.concave[i] = conc[i] != 0;
    p.r = reinterpret_cast<double *>(take(24 * n));
    p.v = reinterpret_cast<double *>(take(24 * n));
    p.vhat = p.v;
    p.mass = reinterpret_cast<double *>(take(8 * n));
    p.dens = reinterpret_cast<double *>(take(8 * n));
    p.h = reinterpret_cast<double *>(take(8 * n));
    p.radius = reinterpret_cast<double *>(take(8 * n));
    p.norm1 = reinterpret_cast<double *>(take(24 * n));
    p.norm2 = reinterpret_cast<double *>(take(24 * n));
    p.norm3 = reinterpret_cast<double *>(take(24 * n));
    return (bool)in;
}

void write_final(const char *path, const particleContainer &ps) {
    std::ofstream out(path, std::ios::binary);
    out.write("SPDMFAC1", 8);
    const int64_t n = (int64_t)ps.size();
    out.write(reinterpret_cast<const char *>(&n), 8);
    for (const Cparticle &q : ps) {
        double rec[14] = {0};
        for (int d = 0; d < NDIM; d++) {
            rec[d] = q.r[d];
            rec[3 + d] = q.v[d];
            rec[6 + d] = q.vhat[d];
            rec[9 + d] = q.f[d];
        }
        rec[12] = q.dens;
        rec[13] = q.h;
        out.write(reinterpret_cast<const char *>(rec), sizeof rec);
    }
}

void fail_exit(sphdem_handle h, const char *what) {
    char msg[512];
    sphdem_last_error(h, msg, sizeof msg);
    std::cerr << what << ": " << msg << std::endl;
    std::exit(-1);
}

void phase(sphdem_handle h, int p, const char *what) {
    if (sphdem_phase(h, p) != SPHDEM_OK) fail_exit(h, what);
}

/* one step of run.cpp:102-118: the case's hooks on the host mirror between
 * the device phases */
void hooked_step(sphdem_handle h, CdataLL &data, CcustomSim &customSim) {
    CglobalVars &globals = data.globals;
    phase(h, SPHDEM_HOOK_BEFORE_START, "step"); /* globals.sphStep++ (run.cpp:104) */
    data.pull();
    customSim.beforeStart(globals.time);
    data.push();
    phase(h, SPHDEM_PHASE_START, "start");
    data.pull();
    customSim.beforeMiddle(globals.time);
    data.push();
    phase(h, SPHDEM_PHASE_MIDDLE, "middle");
    data.pull();
    customSim.beforeEnd(globals.time);
    data.push();
    phase(h, SPHDEM_PHASE_END, "end");
    data.pull();
    customSim.afterEnd(globals.time);
    data.push();
}

/* sph.calcOutputVars() (sphIncompress.h:274-319, run.cpp:131): the
 * output-step quantities into the globals */
void output_vars(sphdem_handle h, CglobalVars &g) {
    SphDemOutputVars ov;
    if (sphdem_output_vars(h, &ov) != SPHDEM_OK) fail_exit(h, "sphdem_output_vars");
    for (int d = 0; d < NDIM; d++) g.linMom[d] = ov.lin_mom[d];
    g.angMom = ov.ang_mom;
    g.eKE = ov.e_ke;
    g.eElast = ov.e_elast;
    g.eElastExact = ov.e_elast_exact;
    g.edElastdt = ov.ed_elast_dt;
    g.eViscF = ov.e_visc_f;
    g.edViscFdt = ov.ed_visc_f_dt;
    g.eFF = ov.e_ff;
    g.edFFdt = ov.ed_ff_dt;
    g.eViscB = ov.e_visc_b;
    g.eBForce = ov.e_b_force;
    g.eTotal = ov.e_total;
    g.maxV = ov.max_v;
    g.maxF = ov.max_f;
    g.maxFF = ov.max_ff;
    g.rmsFF = ov.rms_ff;
    g.aveDens = ov.ave_dens;
    g.varDens = ov.var_dens;
    g.aveDensFromMass = ov.ave_dens_from_mass;
    g.n = (int)ov.n;
    g.nSph = (int)ov.n_sph;
}

bool is_file(const char *path) {
    struct stat st;
    return stat(path, &st) == 0 && S_ISREG(st.st_mode);
}

/* run.cpp:16-164 on one process: read the Domain, Globals row and restart of
 * output step intimestep under inbase, then step and write outputs under
 * outbase until MAXTIME or OUTSTEP */
int run_reference_loop(const std::string &inbase, int intimestep, const std::string &outbase, bool mixed,
                       bool fixed_dt) {
    CglobalVars globals;
    Cio_data_vtk io_data(inbase, &globals);
    if (!io_data.readDomain(intimestep, &globals))
        std::cout << "no Domain file under " << inbase << ": the domain is RMIN..RMAX" << std::endl;
    io_data.readGlobals(intimestep, &globals);
    particleContainer ps0;
    io_data.readRestart(intimestep, &ps0, &globals);
    int outstep = intimestep;
#if defined(TIME_OVERIDE) && defined(START_TIME)
    if (TIME_OVERIDE) globals.time = START_TIME;
#endif
#if defined(NSTEP_OVERIDE) && defined(START_NSTEP)
    if (NSTEP_OVERIDE) outstep = START_NSTEP;
#endif
    io_data.setFilename(outbase, &globals);

    SphDemParticles init;
    std::vector<std::vector<char> > keep;
    soa_of(ps0, init, keep);
    SphDemConfig cfg = sphdem_case_config(mixed ? SPHDEM_PREC_MIXED : SPHDEM_PREC_FP64, fixed_dt);
    for (int d = 0; d < NDIM; d++) {
        /* the binning domain is the process's domain (dataLL.cpp:13-14) */
        cfg.domain_min[d] = globals.procDomain[2 * d];
        cfg.domain_max[d] = globals.procDomain[2 * d + 1];
    }
    sphdem_handle h = nullptr;
    const int64_t capacity = std::max<int64_t>(init.n, MAX_NUM_PARTICLES_PER_CPU);
    if (sphdem_create(&cfg, &init, capacity, &h) != SPHDEM_OK) fail_exit(nullptr, "sphdem_create");
    /* the time and step count of the Globals row, maxdt of run.cpp:87 */
    SphDemGlobals dg;
    if (sphdem_get_globals(h, &dg) != SPHDEM_OK) fail_exit(h, "sphdem_get_globals");
    dg.time = globals.time;
    dg.sph_step = globals.sphStep;
    dg.maxdt = MAXTIME / OUTSTEP;
    if (sphdem_set_globals(h, &dg) != SPHDEM_OK) fail_exit(h, "sphdem_set_globals");

    particleContainer ps((size_t)init.n);
    CdataLL data(ps, globals, h);
    data.pull();
    CcustomSim customSim(&data, globals.time);
    CcustomOutput customOutput(&data);
#ifndef START_WRITE_TIME
    double nextWriteTime = globals.time + MAXTIME / OUTSTEP;
#else
    double nextWriteTime = START_WRITE_TIME;
#endif
    while (globals.time <= MAXTIME && outstep <= OUTSTEP) {
        hooked_step(h, data, customSim);
        if (globals.time >= nextWriteTime) {
            outstep++;
            globals.outstep = outstep;
            output_vars(h, globals);
            customOutput.calcOutput(outstep, &customSim, &io_data);
            io_data.writeOutput(outstep, ps, &globals);
            io_data.writeGlobals(outstep, &globals);
            if (outstep % RESTART_EVERY_N_STEPS == 0) {
                io_data.writeRestart(outstep, ps, &globals);
                io_data.writeDomain(outstep, &globals);
            }
            nextWriteTime = globals.time + MAXTIME / OUTSTEP;
            globals.maxdt = MAXTIME / OUTSTEP;
        }
    }
    sphdem_destroy(h);
    return 0;
}

}  // namespace

int main(int argc, char *argv[]) {
    if (argc < 4) {
        std::cout << "Usage: run_case <inbase> <intimestep> <outbase> [--mixed] [--fixed-dt]\n"
                     "       run_case <initial state> <nsteps> <final state> [--mixed] [--fixed-dt]"
                     " [--restart-out <base>] [--dump-config <file>]"
                  << std::endl;
        return -1;
    }
    bool mixed = false, fixed_dt = false;
    const char *restart_out = nullptr, *dump_config = nullptr;
    for (int i = 4; i < argc; i++) {
        if (!std::strcmp(argv[i], "--mixed")) mixed = true;
        if (!std::strcmp(argv[i], "--fixed-dt")) fixed_dt = true;
        if (!std::strcmp(argv[i], "--restart-out") && i + 1 < argc) restart_out = argv[++i];
        if (!std::strcmp(argv[i], "--dump-config") && i + 1 < argc) dump_config = argv[++i];
    }
    if (const char *why = sphdem_case_unsupported()) {
        std::cerr << "this case cannot run on the device path: " << why << std::endl;
        return -1;
    }
    /* run.cpp's command line: a base name, not a file */
    if (!is_file(argv[1])) return run_reference_loop(argv[1], std::atoi(argv[2]), argv[3], mixed, fixed_dt);
    SphDemParticles init;
    std::vector<std::vector<char> > keep;
    const std::string in_path = argv[1];
    const bool vtk_in = ends_with(in_path, ".vtu") || ends_with(in_path, ".pvtu");
    if (!(vtk_in ? read_vtk_state(in_path, init, keep) : read_state(argv[1], init, keep))) {
        std::cerr << "cannot read " << argv[1] << std::endl;
        return -1;
    }
    const int nsteps = std::atoi(argv[2]);
    SphDemConfig cfg = sphdem_case_config(mixed ? SPHDEM_PREC_MIXED : SPHDEM_PREC_FP64, fixed_dt);
    if (dump_config) {
        std::ofstream dc(dump_config, std::ios::binary);
        dc.write(reinterpret_cast<const char *>(&cfg), sizeof cfg);
    }
    sphdem_handle h = nullptr;
    /* room for the particles the case's hooks insert (dataLL.cpp:241) */
    const int64_t capacity = std::max<int64_t>(init.n, MAX_NUM_PARTICLES_PER_CPU);
    if (sphdem_create(&cfg, &init, capacity, &h) != SPHDEM_OK) fail_exit(nullptr, "sphdem_create");
    CglobalVars globals;
    particleContainer ps((size_t)init.n);
    CdataLL data(ps, globals, h);
    data.pull();
    CcustomSim customSim(&data, globals.time);
    CcustomOutput customOutput(&data);
    Cio_data_vtk io(std::string(argv[3]), &globals);
    int outstep = 0;
    for (int s = 0; s < nsteps; s++) {
        hooked_step(h, data, customSim);
        if ((s + 1) % OUTSTEP == 0) {
            data.pull();
            customOutput.calcOutput(++outstep, &customSim, &io);
        }
    }
    data.pull();
    write_final(argv[3], ps);
    if (restart_out) {
        Cio_data_vtk rio(std::string(restart_out), &globals);
        rio.setExactPoints(true);
        rio.writeRestart(nsteps, ps, &globals);
    }
    sphdem_destroy(h);
    return 0;
}
