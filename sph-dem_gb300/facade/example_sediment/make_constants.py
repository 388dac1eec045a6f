"""Write customConstants.h of the example case from a seeded workload of
sphdem.cases, so that the compile-time constants and the initial state agree.

    python make_constants.py [workload] > customConstants.h
"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
from sphdem import cases  # noqa: E402


def constants(name: str = "sediment3d_small") -> str:
    case = cases.workload(name)
    c = case.cfg
    outstep = 10
    r = lambda v: repr(float(v))  # noqa: E731
    lines = [
        "/* Example SPH-DEM sedimentation case for the device façade (generated by",
        f" * make_constants.py from the `{name}` workload: keep the two in step). */",
        "#ifndef CUSTOMCONSTANTS_H",
        "#define CUSTOMCONSTANTS_H",
        "",
        "#include <cmath>",
        "",
        "#define _3D_",
        "#define NDIM 3",
        "#define WENDLAND",
        "#define VISC_MORRIS",
        "#define VAR_H_CORRECTION",
        "#define LIQ_DEM",
        "#define LINEAR",
        "#define NO_ANTICLUMPING",
        "",
        f"const double PI = {r(c['pi'])};",
        f"const double RMIN[NDIM] = {{{', '.join(r(v) for v in c['rmin'])}}};",
        f"const double RMAX[NDIM] = {{{', '.join(r(v) for v in c['rmax'])}}};",
        f"const int PERIODIC[NDIM] = {{{', '.join(str(int(v)) for v in c['periodic'])}}};",
        "const int GHOST[2*NDIM] = {0, 0, 0, 0, 0, 0};",
        "const double DENS_DROP[NDIM] = {0.0, 0.0, 0.0};",
        f"const double PSEP = {r(c['psep'])};",
        f"const double HFAC = {r(c['hfac'])};",
        f"const double H = {r(c['h'])};",
        f"const double DENS = {r(c['dens'])};",
        f"const double REFD = {r(c['refd'])};",
        f"const double GAMMA = {r(c['gamma'])};",
        f"const double PRB = {r(c['prb'])};",
        f"const double SPSOUND = {r(c['spsound'])};",
        f"const double VISCOSITY = {r(c['viscosity'])};",
        f"const double BFAC = {r(c['bfac'])};",
        f"const int OUTSTEP = {outstep};",
        f"const double MAXTIME = {r(c['maxdt'])} * OUTSTEP;",
        "const int RESTART_EVERY_N_STEPS = 5;",
        "#define TIME_OVERIDE 0",
        "#define START_TIME 0",
        "#define NSTEP_OVERIDE 0",
        "#define START_NSTEP 0",
        f"const double DAMPTIME = {r(c['damptime'])};",
        f"const int MAX_NUM_PARTICLES_PER_CPU = {case.n + 256};",
        f"const int REINIT_DENS_EVERY_N_STEPS = {int(c['reinit_dens_every']) or 50000000};",
        f"const int REINIT_DENS_AT_N_STEPS = {int(c['reinit_dens_at']) or 50000000};",
        f"const double TIME_DROP_PARTICLE = {r(c['time_drop_particle'])};",
        f"const double DEM_RADIUS = {r(c['dem_radius'])};",
        f"const double DEM_DENS = {r(c['dem_dens'])};",
        f"const double DEM_K = {r(c['dem_k'])};",
        f"const double DEM_GAMMA = {r(c['dem_gamma'])};",
        f"const double DEM_VOL = {r(c['dem_vol'])};",
        "const double DEM_MIN_REDUCED_MASS = 0.5 * DEM_VOL * DEM_DENS;",
        f"const double LIQ_DEM_COUPLING_RADIUS = {r(c['coupling_radius'])};",
        "",
        "#endif",
    ]
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    sys.stdout.write(constants(*sys.argv[1:]))
