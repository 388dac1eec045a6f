/*
 * Host-side particle record of the plug-in surface: the fields case hook
 * code reads and writes, mirrored from the device state by CdataLL.  Particle
 * types keep the reference's enumeration values (particle.h iamTypes), which
 * are also the iam codes of the C ABI.
 */
#ifndef SPHDEM_FACADE_PARTICLE_H
#define SPHDEM_FACADE_PARTICLE_H

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
};

typedef vector<Cparticle> particleContainer;

#endif
