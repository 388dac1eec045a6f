/*
 * Step globals visible to case hooks (globalVars.h CglobalVars): time, time
 * step, step count and the custom accumulation buffer, which the façade keeps
 * in sync with the handle's device globals around every hook; the output-step
 * quantities calcOutputVars sets (sphIncompress.h:274-319) and the Globals
 * file rows carry (ioGlobals.cpp:39-46); the processor domain and
 * neighbours of the Domain file (ioDomain.cpp:3-40).  Defaults as the
 * reference's constructor sets them (globalVars.h:13-56): the domain is
 * RMIN..RMAX on every axis.
 */
#ifndef SPHDEM_FACADE_GLOBALVARS_H
#define SPHDEM_FACADE_GLOBALVARS_H

#include "customConstants.h"
#include "vect.h"

#ifndef GLOBAL_CUSTOM_BUFFER_SIZE
#define GLOBAL_CUSTOM_BUFFER_SIZE 9
#endif

/* 3^NDIM: the processor and its neighbours along every axis */
#define SPHDEM_FACADE_NEIGHBOURS (NDIM == 1 ? 3 : (NDIM == 2 ? 9 : 27))

class CglobalVars {
   public:
    CglobalVars() {
        for (int d = 0; d < NDIM; d++) {
            procDomain[2 * d] = RMIN[d];
            procDomain[2 * d + 1] = RMAX[d];
        }
        for (int k = 0; k < SPHDEM_FACADE_NEIGHBOURS; k++) procNeighbrs[k] = -1;
    }

    double time = 0, dt = 0, newDt = 0, maxdt = 0, demDt = 0;
    int sphStep = 0;
    double custom[GLOBAL_CUSTOM_BUFFER_SIZE] = {0};
    int mpiRank = 0, mpiSize = 1;
    int n = 0, nSph = 0;

    /* calcOutputVars */
    double angMom = 0;
    vect linMom = 0.0;
    double eBForce = 0, eElast = 0, eElastExact = 0, eKE = 0, eViscF = 0, eViscB = 0, eFF = 0, eTotal = 0;
    double edElastdt = 0, edViscFdt = 0, edFFdt = 0;
    double maxV = 0, aveDens = 0, varDens = 0, aveDensFromMass = 0;
    double maxF = 0, maxFF = 0, rmsFF = 0;

    /* the Domain file: [min, max] per axis, neighbour ranks (-1: none) */
    double procDomain[NDIM * 2];
    int procNeighbrs[SPHDEM_FACADE_NEIGHBOURS];

    int outstep = 0;
};

#endif
