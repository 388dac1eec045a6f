#include "customSim.h"

#include "dataLL.impl.h"
#include "sph.h"

namespace {

inline void fluidGravity(Cparticle &p, CglobalVars &g) { p.f[2] -= 9.81; }

inline void sphereGravityAndFloor(Cparticle &p, CglobalVars &g) {
    p.f[2] -= 9.81;
    /* spring-dashpot contact with the floor z = RMIN[2] */
    const double overlap = DEM_RADIUS - (p.r[2] - RMIN[2]);
    if (overlap > 0.0) {
        const vect up(0.0, 0.0, 1.0);
        const vect fw = Nsph::demNormal(overlap, -p.vhat[2], up) / p.mass;
        p.fb += fw;
        p.f += fw;
    }
}

}  // namespace

void CcustomSim::beforeMiddle(double newTime) { data->traverse<fluidGravity, Nsph::ifSph>(); }

void CcustomSim::beforeEnd(double newTime) { data->traverse<sphereGravityAndFloor, Nsph::ifDem>(); }
