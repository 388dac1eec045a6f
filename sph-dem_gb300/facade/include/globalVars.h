/*
 * Step globals visible to case hooks (globalVars.h CglobalVars): time, time
 * step, step count and the custom accumulation buffer.  The façade keeps them
 * in sync with the handle's device globals around every hook.
 */
#ifndef SPHDEM_FACADE_GLOBALVARS_H
#define SPHDEM_FACADE_GLOBALVARS_H

#include "customConstants.h"

#ifndef GLOBAL_CUSTOM_BUFFER_SIZE
#define GLOBAL_CUSTOM_BUFFER_SIZE 9
#endif

class CglobalVars {
   public:
    double time = 0, dt = 0, newDt = 0, maxdt = 0, demDt = 0;
    int sphStep = 0;
    double custom[GLOBAL_CUSTOM_BUFFER_SIZE] = {0};
    int mpiRank = 0, mpiSize = 1;
    int n = 0, nSph = 0;
};

#endif
