/* Hooks of the example sedimentation case: gravity on the fluid before the
 * middle phase; gravity and a bottom wall on the DEM spheres before the end
 * phase (the pattern of a sedimentation case's customSim). */
#ifndef CUSTOMSIM_H
#define CUSTOMSIM_H

#include "customConstants.h"
#include "customSimBase.h"
#include "dataLL.h"
#include "sph.h"
#include "vect.h"

class CcustomSim : public CcustomSimBase {
   public:
    CcustomSim(CdataLL *_data, double _time) : CcustomSimBase(_data, _time) {}
    void beforeMiddle(double newTime);
    void beforeEnd(double newTime);
};

#endif
