/*
 * Host-side particle record of the plug-in surface: the fields case hook
 * code reads and writes, mirrored from the device state by CdataLL.  Particle
 * types keep the reference's enumeration values (particle.h iamTypes), which
 * are also the iam codes of the C ABI.
 */
#ifndef SPHDEM_FACADE_PARTICLE_H
#define SPHDEM_FACADE_PARTICLE_H

#include <cmath>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "vect.h"

/* case sources are written against headers that bring in namespace std */
using namespace std;

enum iamTypes {
    sph, sphBoundary, immovable, boundary, ghost,
    boundaryobj1, boundaryobj2, boundaryobj3, boundaryobj4, boundaryobj5, boundaryobj6,
    dem, demBoundary, immersedDem
};

class Cparticle {
   public:
    vect r, v, vhat, v0, vhat0;
    vect f, fp, fv, fb, ff;          /* total, pressure, viscous, boundary, (host-only) */
    vect fdrag, fvel, gradPorosity;
    vect norm1, norm2, norm3;
    double mass = 0, dens = 0, h = 0, dddt = 0, press = 0, pdr2 = 0;
    double porosity = 1, dporositydt = 0, shepSum = 0, omega = 1, radius = 0;
    enum iamTypes iam = sph;
    int tag = 0;
    bool concave = true;
    /* calcEnergies integrals per unit mass (sphIncompress.h:769-781): u, dudt,
     * eViscF and deViscFdt are mirrored from the device; the other three
     * pairs are zero on the device path, as on the reference's */
    double u = 0, dudt = 0;
    double eViscF = 0, deViscFdt = 0, eViscB = 0, deViscBdt = 0, eBForce = 0, deBForcedt = 0, eFF = 0, deFFdt = 0;
    /* members the reference's particle carries for case and output code
     * (particle.h:262-316); host-only here */
    vect fg, vort, origPos;
    double tmp = 0, minDt = 0, colour = 0;
    int gHead = 0;

    /* the neighbour predicate (particle.h:236-238), Wendland support 2h */
    bool is_neighbr(Cparticle &p) {
        return (&p != this) && len2(r - p.r) <= std::pow(2.0 * (h > p.h ? h : p.h), 2);
    }
};

typedef vector<Cparticle> particleContainer;

#endif
