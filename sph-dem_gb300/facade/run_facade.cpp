/*
 * Driver of a case directory on the device (the step loop of run.cpp:80-170):
 * compiled together with the case's customConstants.h, customSim.cpp and
 * customOutput.cpp against the façade headers (include/), linked with
 * libsphdem.so.
 *
 *   run_case <initial state> <nsteps> <final state out> [--mixed] [--fixed-dt]
 *            [--restart-out <base>] [--dump-config <file>]
 *
 * The initial state is a restart piece or index the case's setup writes
 * (<base>Restart0000000_0.vtu / .pvtu, read as Cio_data_vtk::readRestart
 * reads it) or an SPDMST01 state file.  --restart-out writes the final state
 * as <base>Restart%07d (the step count) with Float64 points;
 * --dump-config writes the SphDemConfig the case's constants give (raw
 * struct bytes).
 *
 * Every step calls the case's beforeStart / beforeMiddle / beforeEnd /
 * afterEnd hooks on the host mirror between the device phases
 * (SPHDEM_PHASE_START / MIDDLE / END), and calcOutput every OUTSTEP steps.
 * The final state is written as r, v, vhat, f, dens, h per particle (tag
 * order) after a 16-byte header ("SPDMFAC1", n).
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
    return true;
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

}  // namespace

int main(int argc, char *argv[]) {
    if (argc < 4) {
        std::cout << "Usage: run_case <initial state> <nsteps> <final state> [--mixed] [--fixed-dt]" << std::endl;
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
    if (sphdem_create(&cfg, &init, capacity, &h) != SPHDEM_OK) {
        std::cerr << "sphdem_create failed" << std::endl;
        return -1;
    }
    CglobalVars globals;
    particleContainer ps((size_t)init.n);
    CdataLL data(ps, globals, h);
    data.pull();
    CcustomSim customSim(&data, globals.time);
    CcustomOutput customOutput(&data);
    Cio_data_vtk io(std::string(argv[3]), &globals);
    auto phase = [&](int p, const char *what) {
        if (sphdem_phase(h, p) != SPHDEM_OK) {
            char msg[512];
            sphdem_last_error(h, msg, sizeof msg);
            std::cerr << what << ": " << msg << std::endl;
            std::exit(-1);
        }
    };
    int outstep = 0;
    for (int s = 0; s < nsteps; s++) {
        phase(SPHDEM_HOOK_BEFORE_START, "step");   /* globals.sphStep++ (run.cpp:104) */
        data.pull();
        customSim.beforeStart(globals.time);
        data.push();
        phase(SPHDEM_PHASE_START, "start");
        data.pull();
        customSim.beforeMiddle(globals.time);
        data.push();
        phase(SPHDEM_PHASE_MIDDLE, "middle");
        data.pull();
        customSim.beforeEnd(globals.time);
        data.push();
        phase(SPHDEM_PHASE_END, "end");
        data.pull();
        customSim.afterEnd(globals.time);
        data.push();
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
