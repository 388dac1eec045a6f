"""Build the reference's own hot path as a CPU checker (test infrastructure).

The reference configures a case at compile time through customConstants.h
and customSim.{h,cpp} inside a case directory (damBreak/makefile:14-26).
This recipe writes those three files for one of our seeded workloads into
``oracle/_ref/<case>/`` (git-ignored), then compiles the unmodified reference
sources where they lie -- dataLL.cpp, misc.cpp, vect.cpp, sphIncompress.cpp
-- together with ``ref_driver.cpp`` and the single-rank MPI / abort-on-call
GSL declarations under ``shim/``.  No reference file is copied or patched:
``-std=gnu++11`` is enough to compile sph.h:1572 (``return 0,0,0;``), which
only fails under C++98 null-pointer-constant rules.  VTK is not needed
because io_data_vtk.cpp is not compiled.

Only this container holds the reference sources; the binaries built here are
used to pin the oracle port and to generate the golden fixtures under
``tests/golden/``.

    python oracle/ref/build_ref.py dambreak2d_small [--run]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from oracle.refroot import REF_ROOT as REF_SRC  # noqa: E402
OUT_ROOT = os.path.join(REPO, "oracle", "_ref")
sys.path.insert(0, os.path.join(REPO, "sph-dem_gb300"))

from sphdem import cases  # noqa: E402
from sphdem.state import write_state  # noqa: E402


def _f(x: float) -> str:
    return repr(float(x))


def _arr(xs, n, conv=_f) -> str:
    return "{" + ",".join(conv(x) for x in list(xs)[:n]) + "}"


def customconstants(case: cases.Case) -> str:
    c = case.cfg
    nd = c["ndim"]
    flags = c["flags"]
    lines = [
        "/* generated by oracle/ref/build_ref.py for workload %s */" % case.name,
        "#ifndef CUSTOMCONSTANTS_H", "#define CUSTOMCONSTANTS_H", "#include <cmath>",
        "#define _%dD_" % nd, "#define NDIM %d" % nd, "#define INCOMPRESS",
        "const double PI = %s;" % _f(c["pi"]),
        "const double RMIN[NDIM] = %s;" % _arr(c["rmin"], nd),
        "const double RMAX[NDIM] = %s;" % _arr(c["rmax"], nd),
        "const double BMIN[NDIM] = %s;" % _arr(c["rmin"], nd),
        "const double BMAX[NDIM] = %s;" % _arr(c["rmax"], nd),
        "#define TIME_OVERIDE 0", "#define START_TIME 0",
        "#define NSTEP_OVERIDE 0", "#define START_NSTEP 0",
        "const double GAMMA = %s;" % _f(c["gamma"]),
        "const double HFAC = %s;" % _f(c["hfac"]),
        "const int PERIODIC[NDIM] = %s;" % _arr(c["periodic"], nd, str),
        "const int GHOST[2*NDIM] = %s;" % _arr([0] * 6, 2 * nd, str),
        "const double DENS_DROP[NDIM] = %s;" % _arr([0.0] * 3, nd),
        "const double DENS = %s;" % _f(c["dens"]),
        "const double REFD = %s;" % _f(c["refd"]),
        "#define WENDLAND",
    ]
    vm = c["visc_model"]
    if vm == cases.VISC_ARTIFICIAL:
        lines += ["#define VISC_ARTIFICIAL",
                  "const double ALPHA_ARTIFICIAL = %s;" % _f(c["alpha_artificial"])]
    elif vm == cases.VISC_MONAGHAN:
        lines += ["#define VISC_MONAGHAN"]
    elif vm == cases.VISC_MORRIS:
        lines += ["#define VISC_MORRIS"]
    if flags & cases.F_NO_ANTICLUMPING:
        lines.append("#define NO_ANTICLUMPING")
    if flags & cases.F_CONST_H:
        lines.append("#define CONST_H")
    if flags & cases.F_VAR_H_CORRECTION:
        lines.append("#define VAR_H_CORRECTION")
    if flags & cases.F_CORRECTED_GRADIENT:
        lines.append("#define CORRECTED_GRADIENT")
    if flags & cases.F_DEM_BLOCK:
        lines.append("#define DEM_BLOCK")
    every = int(c.get("reinit_dens_every", 0))
    at = int(c.get("reinit_dens_at", 0))
    n = case.n
    lines += [
        "const int OUTSTEP = 1000000;", "const int RESTART_EVERY_N_STEPS = 1000000;",
        "const int REINIT_DENS_EVERY_N_STEPS = %d;" % (every if every > 0 else 2000000000),
        "const int REINIT_DENS_AT_N_STEPS = %d;" % (at if at > 0 else -1),
        "const double MAXTIME = 1e30;",
        "const double DAMPTIME = %s;" % _f(c["damptime"]),
        "const double VREF = 1.0;", "const double REYNOLDS_NUMBER = 1.0;",
        "const double VMAX = 1.0;",
        "const double VISCOSITY = %s;" % _f(c["viscosity"]),
        "const double CSFAC = 10.0;",
        "const double SPSOUND = %s;" % _f(c["spsound"]),
        "const double PRB = %s;" % _f(c["prb"]),
        "const int NX = 10;", "const int NY = 10;", "const int NZ = 10;",
        "const int MAX_NUM_PARTICLES_PER_CPU = %d;" % (n + case.n_inserted + 64),
        "const double PSEP = %s;" % _f(c["psep"]),
        "const double BFAC = %s;" % _f(c["bfac"]),
        "const double H = %s;" % _f(c["h"]),
        "const double APPROX_SMOOTH_GRID_SIZE = H;", "const double SMOOTH_GRID_SIZE = H;",
        "const double GRIDSEP = PSEP;", "#define MIN_ALPHA 0.1",
        "const double ORACLE_MAXDT = %s;" % _f(c["maxdt"]),
        "const bool ORACLE_FIXED_DT = %s;" % ("true" if flags & cases.F_FIXED_DT else "false"),
    ]
    if flags & cases.F_LIQ_DEM:
        ndem = int((case.particles["iam"] == cases.DEM).sum())
        lines += [
            "#define LIQ_DEM", "#define LINEAR", "#define LIQ_DEM_CUSTOM_WALL_CONTACTS",
            "const double DEM_RADIUS = %s;" % _f(c["dem_radius"]),
            "const double DEM_DENS = %s;" % _f(c["dem_dens"]),
            "const double DEM_K = %s;" % _f(c["dem_k"]),
            "const double DEM_VOL = %s;" % _f(c["dem_vol"]),
            "const double DEM_MASS = DEM_VOL*DEM_DENS;",
            "const double DEM_GAMMA = %s;" % _f(c["dem_gamma"]),
            "const double DEM_MIN_REDUCED_MASS = 0.5*DEM_MASS;",
            "const double POROSITY = 1.0;",
            "const double LIQ_DEM_COUPLING_RADIUS = %s;" % _f(c["coupling_radius"]),
            "const double TIME_DROP_PARTICLE = %s;" % _f(c["time_drop_particle"]),
            "const int MAX_NUM_DEM_PARTICLES = %d;" % (ndem + 64),
        ]
    lines += ["#endif", ""]
    return "\n".join(lines)


CUSTOMSIM_H = """/* generated by oracle/ref/build_ref.py */
#ifndef CUSTOMSIM_H
#define CUSTOMSIM_H
#include "customSimBase.h"
#include "customConstants.h"
#include "dataLL.h"
#include "sph.h"
#include "vect.h"
class CcustomSim : public CcustomSimBase {
   public:
      CcustomSim(CdataLL *_data,double _time): CcustomSimBase(_data,_time) {}
      void beforeStart(double newTime);
      void beforeMiddle(double newTime);
      void beforeEnd(double newTime);
      void afterEnd(double newTime);
};
#endif
"""


def customsim_cpp(case: cases.Case) -> str:
    """Hooks in the reference's own customSim pattern (sediment3D/customSim.cpp):
    gravity on sph in beforeMiddle, gravity + planar walls (+ freeze) on dem
    in beforeEnd, freeze again in afterEnd."""
    c = case.cfg
    nd = c["ndim"]
    walls = c["walls"][: c["n_walls"]]
    lines = [
        "/* generated by oracle/ref/build_ref.py for workload %s */" % case.name,
        '#include "customSim.h"', '#include "sph.h"', '#include "dataLL.impl.h"',
        "static const double GSPH[3] = %s;" % _arr(c["gravity_sph"], 3),
        "static const double GDEM[3] = %s;" % _arr(c["gravity_dem"], 3),
        "static const int NWALLS = %d;" % len(walls),
        "static const double WALLP[%d][3] = {%s};" % (max(1, len(walls)), ",".join(
            _arr(w["point"], 3) for w in walls) or "{0,0,0}"),
        "static const double WALLN[%d][3] = {%s};" % (max(1, len(walls)), ",".join(
            _arr(w["normal"], 3) for w in walls) or "{0,0,0}"),
        "static const double FREEZE_UNTIL = %s;" % _f(c["freeze_dem_until"]),
        "inline void addGravitySph(Cparticle &p,CglobalVars &g) {",
        "   for (int i=0;i<NDIM;i++) if (GSPH[i]!=0.0) p.f[i] += GSPH[i];", "}",
        "inline void addGravityDem(Cparticle &p,CglobalVars &g) {",
        "   for (int i=0;i<NDIM;i++) if (GDEM[i]!=0.0) p.f[i] += GDEM[i];", "}",
    ]
    if c["flags"] & cases.F_LIQ_DEM:
        lines += [
            "inline void addWalls(Cparticle &p,CglobalVars &g) {",
            "   for (int w=0;w<NWALLS;w++) {",
            "      vect pt, nn;",
            "      for (int i=0;i<NDIM;i++) { pt[i] = WALLP[w][i]; nn[i] = WALLN[w][i]; }",
            "      const double overlap = DEM_RADIUS - dot(p.r-pt,nn);",
            "      if (overlap>0.0) {",
            "         const double overlap_dot = -dot(p.vhat,nn);",
            "         const vect fNorm = Nsph::demNormal(overlap,overlap_dot,nn)/p.mass;",
            "         p.fb += fNorm;", "         p.f += fNorm;", "      }", "   }", "}",
            "inline void freezeDem(Cparticle &p,CglobalVars &g) {",
            "   p.f = 0.0; p.v = 0.0; p.vhat = p.v;", "}",
        ]
    lines += [
        "void CcustomSim::beforeStart(double newTime) {}",
        "void CcustomSim::beforeMiddle(double newTime) {",
        "   data->traverse<addGravitySph,Nsph::ifSph>();", "}",
        "void CcustomSim::beforeEnd(double newTime) {",
    ]
    if c["flags"] & cases.F_LIQ_DEM:
        lines += [
            "   data->traverse<addGravityDem,Nsph::ifDem>();",
            "   data->traverse<addWalls,Nsph::ifDem>();",
            "   if (data->globals.time <= FREEZE_UNTIL) data->traverse<freezeDem,Nsph::ifDem>();",
        ]
    lines += ["}", "void CcustomSim::afterEnd(double newTime) {"]
    if c["flags"] & cases.F_LIQ_DEM:
        lines += ["   if (data->globals.time <= FREEZE_UNTIL) data->traverse<freezeDem,Nsph::ifDem>();"]
    lines += ["}", ""]
    return "\n".join(lines)


def build(case: cases.Case, opt: str = "-O2") -> str:
    """Write the case files and compile; returns the driver path."""
    if not os.path.isdir(REF_SRC):
        raise FileNotFoundError("reference sources not present: " + REF_SRC)
    d = os.path.join(OUT_ROOT, case.name)
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "customConstants.h"), "w") as fh:
        fh.write(customconstants(case))
    with open(os.path.join(d, "customSim.h"), "w") as fh:
        fh.write(CUSTOMSIM_H)
    with open(os.path.join(d, "customSim.cpp"), "w") as fh:
        fh.write(customsim_cpp(case))
    exe = os.path.join(d, "ref_driver")
    srcs = [os.path.join(REF_SRC, s) for s in
            ("dataLL.cpp", "misc.cpp", "vect.cpp", "sphIncompress.cpp")]
    srcs += [os.path.join(d, "customSim.cpp"), os.path.join(HERE, "ref_driver.cpp")]
    cmd = ["g++", "-std=gnu++11", opt, "-ffp-contract=off", "-fpermissive", "-w",
           "-I" + d, "-I" + os.path.join(HERE, "shim"), "-I" + REF_SRC,
           *srcs, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def run(case: cases.Case, nsteps: int | None = None, exe: str | None = None) -> str:
    """Run the built driver on the case's initial state; returns the output path."""
    d = os.path.join(OUT_ROOT, case.name)
    exe = exe or os.path.join(d, "ref_driver")
    state = os.path.join(d, "init.state")
    out = os.path.join(d, "out.bin")
    write_state(state, case.particles, case.events)
    steps = case.nsteps if nsteps is None else nsteps
    res = subprocess.run([exe, state, out, str(steps)], capture_output=True, text=True)
    sys.stderr.write(res.stderr)
    if res.returncode not in (0,):
        raise RuntimeError(f"ref_driver exited {res.returncode}: {res.stderr[-2000:]}")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload")
    ap.add_argument("--run", action="store_true")
    ap.add_argument("--steps", type=int, default=None)
    a = ap.parse_args()
    case = cases.workload(a.workload)
    exe = build(case)
    print(exe)
    if a.run:
        print(run(case, a.steps))


if __name__ == "__main__":
    main()
