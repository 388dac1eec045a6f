/*
 * Nsph helpers case hook and output code calls (sph.h): the particle-type
 * predicates (sph.h:1827-1889, with the reference's bodies, including
 * ifDemOrDemBoundary testing dem only and ifSphOrSphBoundaryOrImmersedDem
 * testing sph and sphBoundary only), the Wendland C2 kernel K, W and its
 * gradient factor F (sph.h:74-80, 199-205, 306-308, written as the
 * reference writes them so that hook arithmetic rounds alike), gradW
 * (sph.h:322-342), calcHFromDens and calcDensity (sph.h:1149-1190, 1823-1825)
 * and the linear DEM normal force (LINEAR, sph.h:1495-1516).  The device
 * implements the step itself.
 */
#ifndef SPH_H
#define SPH_H

#include <cmath>
#include <vector>

#include "customConstants.h"
#include "demConstants.h"
#include "globalVars.h"
#include "particle.h"
#include "vect.h"

namespace Nsph {

inline bool ifSph(Cparticle &p) { return p.iam == sph; }
inline bool ifDem(Cparticle &p) { return p.iam == dem; }
inline bool ifGhost(Cparticle &p) { return p.iam == ghost; }
inline bool ifDemOrGhost(Cparticle &p) { return p.iam == dem || p.iam == ghost; }
inline bool ifDemOrDemBoundary(Cparticle &p) { return p.iam == dem; }
inline bool ifSphOrDem(Cparticle &p) { return p.iam == sph || p.iam == dem; }
inline bool ifSphOrBoundary(Cparticle &p) { return p.iam == sph || p.iam == boundary; }
inline bool ifSphOrSphBoundaryOrBoundary(Cparticle &p) {
    return p.iam == sph || p.iam == boundary || p.iam == sphBoundary;
}
inline bool ifSphOrDemOrDemBoundary(Cparticle &p) { return p.iam == sph || p.iam == dem || p.iam == demBoundary; }
inline bool ifSphOrSphBoundaryOrDemOrDemBoundary(Cparticle &p) {
    return p.iam == sph || p.iam == sphBoundary || p.iam == dem || p.iam == demBoundary;
}
inline bool ifSphBoundary(Cparticle &p) { return p.iam == sphBoundary; }
inline bool ifSphOrSphBoundary(Cparticle &p) { return p.iam == sph || p.iam == sphBoundary; }
inline bool ifSphOrSphBoundaryOrImmersedDem(Cparticle &p) { return p.iam == sph || p.iam == sphBoundary; }
inline bool ifSphOrSphBoundaryOrDem(Cparticle &p) { return p.iam == sph || p.iam == sphBoundary || p.iam == dem; }
inline bool ifSphOrSphBoundaryOrImmersedDemOrDem(Cparticle &p) {
    return p.iam == sph || p.iam == sphBoundary || p.iam == dem;
}
inline bool ifSphOrSphBoundaryOrGhost(Cparticle &p) { return p.iam == sph || p.iam == sphBoundary || p.iam == ghost; }
inline bool ifSphOrSphBoundaryOrImmersedDemOrGhost(Cparticle &p) {
    return p.iam == sph || p.iam == sphBoundary || p.iam == ghost;
}
inline bool ifSphOrSphBoundaryOrDemOrGhost(Cparticle &p) {
    return p.iam == sph || p.iam == sphBoundary || p.iam == dem || p.iam == ghost;
}
inline bool ifSphOrGhost(Cparticle &p) { return p.iam == sph || p.iam == ghost; }
inline bool ifBoundary(Cparticle &p) {
    return p.iam == boundary || (p.iam >= boundaryobj1 && p.iam <= boundaryobj6);
}
inline bool ifBoundaryOrSphBoundary(Cparticle &p) { return p.iam == boundary || p.iam == sphBoundary; }

/* Wendland C2 normalisation (2D, 3D), support q <= 2 */
const double WCON_WENDLAND = NDIM == 2 ? 7.0 / (64.0 * PI) : 21.0 / (256.0 * PI);

inline double K(const double q, const double h) {
    if (q <= 2.0) return WCON_WENDLAND * std::pow(2.0 - q, 4) * (1.0 + 2.0 * q);
    return 0.0;
}
inline double W(const double q, const double h) { return (1 / std::pow(h, NDIM)) * K(q, h); }
/* dW/dr / r */
inline double F(const double q, const double h) {
    if (q <= 2.0)
        return (1 / std::pow(h, NDIM + 2)) * WCON_WENDLAND *
               (-4 * std::pow(2 - q, 3) * (1 + 2 * q) + 2 * std::pow(2 - q, 4)) / q;
    return 0.0;
}

#ifdef CORRECTED_GRADIENT
/* The corrected gradient reads each particle's invM, sumGrad and sum, which
 * the device computes and keeps to itself: case code that calls gradW under
 * CORRECTED_GRADIENT does not compile against the host mirror. */
template <typename P>
inline vect gradW(const P &, const P &, const vect, const double, const double) {
    static_assert(sizeof(P) == 0, "gradW under CORRECTED_GRADIENT needs invM, which the host mirror does not hold");
    return vect(0.0);
}
#else
inline vect gradW(const Cparticle &pa, const Cparticle &pb, const vect dr, const double q, const double h) {
    vect drF = 0.0;
    if (q != 0) drF = dr * F(q, h);
#ifdef VAR_H_CORRECTION
    return drF / pa.omega;
#else
    (void)pb;
    return drF;
#endif
}
#endif

inline void calcHFromDens(Cparticle &p, CglobalVars &) { p.h = HFAC * std::pow(p.mass / p.dens, 1.0 / NDIM); }

/* the SPH density summation with the particle's own h, over the sph and
 * sphBoundary particles of its neighbour group */
inline void calcDensity(Cparticle &p, std::vector<Cparticle *> &neighbrs, CglobalVars &) {
    p.dens = p.mass * W(0, p.h);
    for (size_t i = 0; i < neighbrs.size(); i++) {
        Cparticle *pn = neighbrs[i];
        if (pn->iam != sph && pn->iam != sphBoundary) continue;
        const vect dr = p.r - pn->r;
        const double r = len(dr);
        p.dens += pn->mass * W(r / p.h, p.h);
    }
}

#ifdef LIQ_DEM
/* linear spring-dashpot normal force magnitude times the normal */
inline vect demNormal(const double overlap, const double overlap_dot, const vect normal) {
    return (DEM_K * overlap + DEM_GAMMA * overlap_dot) * normal;
}
#endif

}  // namespace Nsph

#endif
