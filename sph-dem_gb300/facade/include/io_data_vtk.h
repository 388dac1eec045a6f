/*
 * Output handle passed to a case's calcOutput.  The VTK restart formats are
 * not part of this build: the façade records output requests only.
 */
#ifndef SPHDEM_FACADE_IO_DATA_VTK_H
#define SPHDEM_FACADE_IO_DATA_VTK_H

#include <string>

#include "globalVars.h"

class Cio_data_vtk {
   public:
    Cio_data_vtk() {}
    Cio_data_vtk(const std::string &fn, CglobalVars *) : filename(fn) {}
    void setFilename(const std::string &fn, CglobalVars *) { filename = fn; }
    std::string filename;
};

#endif
