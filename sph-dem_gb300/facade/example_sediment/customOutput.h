/* Output of the example case: mean height of the DEM spheres per output step. */
#ifndef CUSTOMOUTPUT_H
#define CUSTOMOUTPUT_H

#include "customConstants.h"
#include "customOutputBase.h"
#include "customSim.h"

class CcustomOutput : public CcustomOutputBase {
   public:
    CcustomOutput(CdataLL *_data) : CcustomOutputBase(_data) {}
    void calcOutput(int outstep, CcustomSim *custSim, Cio_data_vtk *io);
};

#endif
