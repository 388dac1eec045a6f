/*
 * Base of a case's CcustomOutput (customOutputBase.h): calcOutput is called by
 * the façade driver every output step with the host mirror current.
 */
#ifndef CUSTOMOUTPUTBASE_H
#define CUSTOMOUTPUTBASE_H

#include "customConstants.h"
#include "customSim.h"
#include "dataLL.h"
#include "io_data_vtk.h"
#include "vect.h"

class CcustomOutputBase {
   public:
    CcustomOutputBase(CdataLL *_data) : data(_data) {}
    virtual ~CcustomOutputBase() {}
    virtual void calcOutput(int outstep, CcustomSim *custSim, Cio_data_vtk *io) {}

   protected:
    CdataLL *data;
};

#endif
