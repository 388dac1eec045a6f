/*
 * Nsph helpers case hook code calls (sph.h): particle-type predicates, the
 * Wendland C2 kernel W(q, h) = h^-d K(q), and the linear DEM normal force
 * (LINEAR, sph.h:1495-1516).  The device implements the step itself.
 */
#ifndef SPH_H
#define SPH_H

#include <cmath>

#include "customConstants.h"
#include "demConstants.h"
#include "globalVars.h"
#include "particle.h"
#include "vect.h"

namespace Nsph {

inline bool ifSph(Cparticle &p) { return p.iam == sph; }
inline bool ifDem(Cparticle &p) { return p.iam == dem; }
inline bool ifSphBoundary(Cparticle &p) { return p.iam == sphBoundary; }
inline bool ifBoundary(Cparticle &p) {
    return p.iam == boundary || (p.iam >= boundaryobj1 && p.iam <= boundaryobj6);
}
inline bool ifSphOrDem(Cparticle &p) { return p.iam == sph || p.iam == dem; }
inline bool ifSphOrBoundary(Cparticle &p) { return p.iam == sph || ifBoundary(p); }
inline bool ifSphOrSphBoundary(Cparticle &p) { return p.iam == sph || p.iam == sphBoundary; }
inline bool ifSphOrSphBoundaryOrDem(Cparticle &p) { return ifSphOrSphBoundary(p) || p.iam == dem; }
inline bool ifDemOrDemBoundary(Cparticle &p) { return p.iam == dem || p.iam == demBoundary; }

/* Wendland C2, support q <= 2 */
inline double K(const double q, const double h) {
    if (q > 2.0) return 0.0;
    const double c = NDIM == 2 ? 7.0 / (64.0 * PI) : 21.0 / (256.0 * PI);
    const double t = 2.0 - q;
    return c * t * t * t * t * (1.0 + 2.0 * q);
}
inline double W(const double q, const double h) { return K(q, h) / std::pow(h, NDIM); }

#ifdef LIQ_DEM
/* linear spring-dashpot normal force magnitude times the normal */
inline vect demNormal(const double overlap, const double overlap_dot, const vect normal) {
    return (DEM_K * overlap + DEM_GAMMA * overlap_dot) * normal;
}
#endif

}  // namespace Nsph

#endif
