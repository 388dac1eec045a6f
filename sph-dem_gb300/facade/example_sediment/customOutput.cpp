#include "customOutput.h"

#include "dataLL.impl.h"
#include "sph.h"

namespace {

inline void sumHeight(Cparticle &p, CglobalVars &g) {
    g.custom[0] += p.r[2];
    g.custom[1] += 1.0;
}

}  // namespace

void CcustomOutput::calcOutput(int outstep, CcustomSim *custSim, Cio_data_vtk *io) {
    data->globals.custom[0] = data->globals.custom[1] = 0.0;
    data->traverse<sumHeight, Nsph::ifDem>();
    std::ofstream fo(io->filename + ".heights", std::ios::app);
    fo << data->globals.time << ' ' << data->globals.custom[0] / data->globals.custom[1] << std::endl;
}
